"""The bounded device waits' expiry path, made to run out on purpose.

Every mbarrier wait of the mixed-precision kernels is bounded; when one runs
out the kernel sets a status word, the other roles leave their loops, TMEM
is released and the C-ABI reports FEM_ERR_TIMEOUT.  fem_em_selftest_wait_
expiry runs a kernel with those roles whose producer never delivers and a
short budget (1e5 cycles, ~50 us): nothing faults or hangs, the waits give up
and the handle keeps working afterwards (the next sweeps allocate the same
512 TMEM columns and match the oracle)."""
import ctypes

import numpy as np
import pytest

from fastem_gb300 import CudaMatrixEM, GaussianMixture, synth
from fastem_gb300 import _capi as C

pytestmark = pytest.mark.gpu


def test_bounded_wait_expiry_reports_timeout_and_recovers(gpu_lib, oracle):
    n, k = 1 << 12, 4
    X, _ = synth.em_large(seed=3, n=n, d=64, k=k)
    init = synth.forgy_init(X, k, seed=1)
    ref = oracle.em_train(X, *init, 2, eps=0.0)
    with CudaMatrixEM(64, n, k, precision="mixed") as em:
        em.CopyDataset(X)
        for _ in range(2):                      # twice: the status word is cleared between calls
            roles = ctypes.c_int(0)
            st = C.lib().fem_em_selftest_wait_expiry(em.handle, 100000, ctypes.byref(roles))
            assert st == C.FEM_ERR_TIMEOUT
            assert b"timed out" in C.lib().fem_last_error()
            # the consumer's and the drain's own budgets ran out; both waiters
            # off the critical path left on the status word
            assert roles.value == 0b1111, bin(roles.value)
        em.SetParameters(2, 0.0, 1e5)
        G = GaussianMixture(*init)
        em.TrainNoCopy(G)
        err = np.abs(em.logl_trace - ref["logl"]) / n
        assert err.max() <= 1e-5, err


def test_bounded_wait_selftest_arguments(gpu_lib):
    roles = ctypes.c_int(0)
    with CudaMatrixEM(64, 1000, 2, precision="fp32") as em:
        assert C.lib().fem_em_selftest_wait_expiry(em.handle, 100000, ctypes.byref(roles)) == C.FEM_ERR_UNSUPPORTED
    with CudaMatrixEM(64, 1000, 2, precision="mixed") as em:
        assert C.lib().fem_em_selftest_wait_expiry(em.handle, 10, ctypes.byref(roles)) == C.FEM_ERR_BAD_ARG
        assert C.lib().fem_em_selftest_wait_expiry(em.handle, 100000, None) == C.FEM_ERR_BAD_ARG
