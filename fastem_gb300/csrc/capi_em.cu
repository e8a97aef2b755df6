// capi_em.cu -- the EM half of the C-ABI (include/fastem_gpu.h).
//
// The sweep loop of EMAlgorithm::TrainNoCopy (EM2/EMAlgorithm.cpp:139-191)
// runs here on the host; each sweep enqueues the E-step, M-step and
// factorisation kernels on the handle's stream and synchronises once to read
// LogL and the factorisation status.
#include <algorithm>
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "em_kernels.cuh"
#include "fem_internal.cuh"

using namespace fem;

void fem::timing_begin(fem_em *h, int slot) {
  if (h->timing) {
    cudaEventRecord(h->ev[slot], h->stream);
    h->tmask |= 1u << slot;
  }
}

namespace {

int check_handle(fem_em *h) {
  if (!h) {
    set_error("null EM handle");
    return FEM_ERR_BAD_ARG;
  }
  return FEM_OK;
}

bool mixed(const fem_em *h) { return h->cfg.precision == FEM_PREC_MIXED; }

// reads the device status word; FEM_ERR_CHOLESKY if a factorisation failed
int sync_status(fem_em *h) {
  FEM_CUDA(cudaMemcpyAsync(h->hstat, h->dstat, sizeof(DevStatus), cudaMemcpyDeviceToHost, h->stream));
  FEM_CUDA(cudaStreamSynchronize(h->stream));
  if (h->timing) {
    float ms = 0;
    double *acc[5] = {&h->t_estep, &h->t_mstep, &h->t_final, nullptr, &h->t_cov};
    for (int p = 0; p < 5; p++) {
      const unsigned both = 3u << (2 * p);
      if (acc[p] && (h->tmask & both) == both &&
          cudaEventElapsedTime(&ms, h->ev[2 * p], h->ev[2 * p + 1]) == cudaSuccess)
        *acc[p] += ms;
    }
    h->tmask = 0;
  }
  if (h->hstat->timeout) {
    set_error("a bounded device wait timed out in the mixed-precision kernels");
    return FEM_ERR_TIMEOUT;
  }
  if (h->hstat->chol_failed != INT_MAX) {
    set_error("Cholesky decomposition failed (component %d)", h->hstat->chol_failed);
    return FEM_ERR_CHOLESKY;
  }
  return FEM_OK;
}

int reset_status(fem_em *h) {
  DevStatus s{};
  s.chol_failed = INT_MAX;
  *h->hstat = s;
  FEM_CUDA(cudaMemcpyAsync(h->dstat, h->hstat, sizeof(DevStatus), cudaMemcpyHostToDevice, h->stream));
  if (mixed(h) && (h->tc || h->wide)) FEM_TRY(em_tc_reset_err(h));
  return FEM_OK;
}

// RegularizeCovariances + InitDensities, enqueued (no sync)
int enqueue_factor(fem_em *h) {
  timing_begin(h, 4);
  FEM_TRY(em_factor(h, true));
  if (mixed(h)) FEM_TRY(em_tc_prepare(h));
  timing_begin(h, 5);
  h->factored = true;
  return FEM_OK;
}

int enqueue_estep(fem_em *h) {
  timing_begin(h, 0);
  FEM_TRY(mixed(h) ? em_tc_estep(h) : em_plain_estep(h));
  timing_begin(h, 1);
  h->have_post = true;
  return FEM_OK;
}

int enqueue_mstep(fem_em *h) {
  timing_begin(h, 2);
  FEM_TRY(mixed(h) ? em_tc_mstep(h) : em_plain_mstep(h));
  timing_begin(h, 3);
  return FEM_OK;
}

int max_cond(fem_em *h, double *cond) { return em_max_cond(h, cond); }

// The condition test of TrainNoCopy (EM2/EMAlgorithm.cpp:147-151,157-161):
// the factorisation just synchronised left max_j ||Sigma_j||_F ||L_j^-1||_F^2,
// an upper bound of every cond(Sigma_j), in the status word.  When that bound
// is within AbortThr no condition number can exceed it, and *cond receives the
// bound; otherwise the exact eigenvalues are computed (k_cond_jacobi) and
// *cond is the largest condition number, as FindLargestConditionNumber.
int cond_check(fem_em *h, double *cond) {
  const double b = h->hstat->cond_bound * (1.0 + 1e-12);
  if (b > 0.0 && b <= h->cfg.abort_thr) {
    *cond = b;
    return FEM_OK;
  }
  return max_cond(h, cond);
}

void free_all(fem_em *h) {
  if (h->tc || h->wide) em_tc_destroy(h);
  dfree(h->X);
  dfree(h->Xhi);
  dfree(h->Xlo);
  dfree(h->pi);
  dfree(h->mu);
  dfree(h->sigma);
  dfree(h->linv);
  dfree(h->logdet);
  dfree(h->logc);
  dfree(h->work);
  if (h->muT) cudaFree(h->muT);
  if (h->linvT) cudaFree(h->linvT);
  if (h->logcT) cudaFree(h->logcT);
  if (h->R) cudaFree(h->R);
  h->muT = h->linvT = h->logcT = h->R = nullptr;
  dfree(h->logl_part);
  dfree(h->mpart);
  dfree(h->cpart);
  dfree(h->psum);
  dfree(h->dstat);
  if (h->hstat) cudaFreeHost(h->hstat);
  h->hstat = nullptr;
  for (auto &e : h->ev)
    if (e) cudaEventDestroy(e), e = nullptr;
  if (h->stream) cudaStreamDestroy(h->stream);
  h->stream = nullptr;
}

}  // namespace

extern "C" {

void fem_em_config_default(fem_em_config *cfg) {
  if (!cfg) return;
  cfg->precision = FEM_PREC_MIXED;
  cfg->device = 0;
  cfg->max_sweeps = 1000000;
  cfg->eps = 1e-5;
  cfg->abort_thr = 1e5;
  cfg->reg_coef = 0.0;
  cfg->svd = 1;
}

int fem_em_create(int d, int64_t n, int k, const fem_em_config *cfg, fem_em **out) {
  if (!out) {
    set_error("out is NULL");
    return FEM_ERR_BAD_ARG;
  }
  *out = nullptr;
  fem_em_config c;
  if (cfg)
    c = *cfg;
  else
    fem_em_config_default(&c);
  if (d < 1 || d > 256 || n < 1 || k < 1 || k > 4096) {
    set_error("bad sizes d=%d n=%lld k=%d (1<=d<=256, n>=1, 1<=k<=4096)", d, (long long)n, k);
    return FEM_ERR_BAD_ARG;
  }
  if (c.precision < FEM_PREC_FP64 || c.precision > FEM_PREC_MIXED) {
    set_error("unknown precision %d", c.precision);
    return FEM_ERR_BAD_ARG;
  }
  if (c.precision == FEM_PREC_MIXED && !em_tc_supported(d, k)) {
    set_error("mixed precision (tensor-core kernels) needs d <= 64 and k <= 128, or 64 < d <= 256 "
              "(got d=%d k=%d); use FEM_PREC_FP32 or FEM_PREC_FP64", d, k);
    return FEM_ERR_UNSUPPORTED;
  }
  FEM_TRY(select_device(c.device));
  fem_em *h = new (std::nothrow) fem_em();
  if (!h) {
    set_error("out of host memory");
    return FEM_ERR_BAD_ARG;
  }
  h->d = d;
  h->n = n;
  h->k = k;
  h->cfg = c;
  auto fail = [&](int st) {
    free_all(h);
    delete h;
    return st;
  };
  if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
    set_error("cudaStreamCreate failed");
    return fail(FEM_ERR_CUDA);
  }
  for (auto &e : h->ev)
    if (cudaEventCreate(&e) != cudaSuccess) return fail(FEM_ERR_CUDA);
  const size_t ts = (c.precision == FEM_PREC_FP64) ? sizeof(double) : sizeof(float);
  const size_t kd = (size_t)k * d, kdd = kd * d;
  int st = FEM_OK;
  if ((st = dalloc(&h->X, (size_t)n * d)) || (st = dalloc(&h->pi, k)) || (st = dalloc(&h->mu, kd)) ||
      (st = dalloc(&h->sigma, kdd)) || (st = dalloc(&h->linv, kdd)) || (st = dalloc(&h->logdet, k)) ||
      (st = dalloc(&h->logc, k)) || (st = dalloc(&h->work, kdd)) || (st = dalloc(&h->psum, k)) ||
      (st = dalloc(&h->dstat, 1)))
    return fail(st);
  // posteriors: k x n in T for the CUDA-core forms; the mixed form keeps FP16 hi/lo pairs
  const size_t rbytes = (c.precision == FEM_PREC_MIXED) ? 0 : (size_t)k * n * ts;
  if (cudaMalloc(&h->muT, kd * ts) != cudaSuccess || cudaMalloc(&h->linvT, kdd * ts) != cudaSuccess ||
      cudaMalloc(&h->logcT, k * ts) != cudaSuccess ||
      (rbytes && cudaMalloc(&h->R, rbytes) != cudaSuccess)) {
    set_error("cudaMalloc failed for the %zu-byte posterior matrix or factors", (size_t)k * n * ts);
    return fail(FEM_ERR_CUDA);
  }
  if (cudaMallocHost(&h->hstat, sizeof(DevStatus)) != cudaSuccess) {
    set_error("cudaMallocHost failed");
    return fail(FEM_ERR_CUDA);
  }
  if (c.precision == FEM_PREC_MIXED) {
    st = em_tc_create(h);
    if (st) return fail(st);
    if (em_tc_small_components(n, k, d)) {
      // partials of the FP32 CUDA-core covariance used for small components
      int TB, nb, nblk;
      cov_geometry(d, &TB, &nb, &nblk);
      const int gx = (k * nblk + 255) / 256;
      h->cchunks = (int)std::max<int64_t>(1, std::min<int64_t>((3 * sm_count() + gx - 1) / gx, (n + 31) / 32));
      if ((st = dalloc(&h->cpart, (size_t)h->cchunks * k * nblk * TB * TB))) return fail(st);
    }
  } else {
    h->n_logl_part = em_plain_logl_blocks(n, d);
    if ((st = dalloc(&h->logl_part, h->n_logl_part))) return fail(st);
    h->mgrid = (int)std::min<int64_t>((int64_t)4 * sm_count(), (n + 31) / 32);
    if ((st = dalloc(&h->mpart, (size_t)h->mgrid * k * (d + 1)))) return fail(st);
    int TB, nb, nblk;
    cov_geometry(d, &TB, &nb, &nblk);
    const int gx = (k * nblk + 255) / 256;
    h->cchunks = (int)std::max<int64_t>(1, std::min<int64_t>((3 * sm_count() + gx - 1) / gx, (n + 31) / 32));
    if ((st = dalloc(&h->cpart, (size_t)h->cchunks * k * nblk * TB * TB))) return fail(st);
  }
  if (reset_status(h)) return fail(FEM_ERR_CUDA);
  *out = h;
  return FEM_OK;
}

void fem_em_destroy(fem_em *h) {
  if (!h) return;
  if (h->stream) cudaStreamSynchronize(h->stream);
  free_all(h);
  delete h;
}

int fem_em_set_parameters(fem_em *h, int max_sweeps, double eps, double abort_thr, double reg_coef) {
  FEM_TRY(check_handle(h));
  if (max_sweeps < 0 || !(eps >= 0.0) || !(reg_coef >= 0.0 && reg_coef <= 1.0)) {
    set_error("bad parameters");
    return FEM_ERR_BAD_ARG;
  }
  h->cfg.max_sweeps = max_sweeps;
  h->cfg.eps = eps;
  h->cfg.abort_thr = abort_thr;
  h->cfg.reg_coef = reg_coef;
  return FEM_OK;
}

static int upload_common(fem_em *h, const float *X, int64_t ld, cudaMemcpyKind kind) {
  FEM_TRY(check_handle(h));
  if (!X || ld < h->d) {
    set_error("bad dataset pointer or ld");
    return FEM_ERR_BAD_ARG;
  }
  FEM_CUDA(cudaSetDevice(h->cfg.device));
  if (ld == h->d)   // contiguous rows: one linear copy
    FEM_CUDA(cudaMemcpyAsync(h->X, X, (size_t)h->n * h->d * sizeof(float), kind, h->stream));
  else
    FEM_CUDA(cudaMemcpy2DAsync(h->X, (size_t)h->d * sizeof(float), X, (size_t)ld * sizeof(float),
                               (size_t)h->d * sizeof(float), (size_t)h->n, kind, h->stream));
  if (mixed(h)) FEM_TRY(em_tc_upload(h));
  FEM_CUDA(cudaStreamSynchronize(h->stream));
  h->have_data = true;
  h->have_post = false;
  return FEM_OK;
}

int fem_em_upload(fem_em *h, const float *X, int64_t ld) {
  return upload_common(h, X, ld, cudaMemcpyHostToDevice);
}

int fem_em_upload_device(fem_em *h, const float *dX, int64_t ld) {
  return upload_common(h, dX, ld, cudaMemcpyDeviceToDevice);
}

int fem_em_set_params(fem_em *h, const double *pi, const double *mu, const double *sigma) {
  FEM_TRY(check_handle(h));
  if (!pi || !mu || !sigma) {
    set_error("null parameter array");
    return FEM_ERR_BAD_ARG;
  }
  FEM_CUDA(cudaSetDevice(h->cfg.device));
  const size_t kd = (size_t)h->k * h->d;
  FEM_CUDA(cudaMemcpyAsync(h->pi, pi, h->k * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  FEM_CUDA(cudaMemcpyAsync(h->mu, mu, kd * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  FEM_CUDA(cudaMemcpyAsync(h->sigma, sigma, kd * h->d * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  FEM_CUDA(cudaStreamSynchronize(h->stream));
  h->have_params = true;
  h->factored = false;
  return FEM_OK;
}

int fem_em_get_params(fem_em *h, double *pi, double *mu, double *sigma) {
  FEM_TRY(check_handle(h));
  if (!h->have_params) {
    set_error("no parameters set");
    return FEM_ERR_STATE;
  }
  const size_t kd = (size_t)h->k * h->d;
  if (pi) FEM_CUDA(cudaMemcpyAsync(pi, h->pi, h->k * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  if (mu) FEM_CUDA(cudaMemcpyAsync(mu, h->mu, kd * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  if (sigma)
    FEM_CUDA(cudaMemcpyAsync(sigma, h->sigma, kd * h->d * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  FEM_CUDA(cudaStreamSynchronize(h->stream));
  return FEM_OK;
}

int fem_em_init_densities(fem_em *h, int *failed) {
  FEM_TRY(check_handle(h));
  if (failed) *failed = -1;
  if (!h->have_params) {
    set_error("no parameters set");
    return FEM_ERR_STATE;
  }
  FEM_TRY(reset_status(h));
  FEM_TRY(enqueue_factor(h));
  int st = sync_status(h);
  if (st == FEM_ERR_CHOLESKY) {
    h->factored = false;
    if (failed) *failed = h->hstat->chol_failed;
  }
  return st;
}

int fem_em_precompute(fem_em *h, double *logl) {
  FEM_TRY(check_handle(h));
  if (!h->have_data || !h->factored) {
    set_error("precompute needs an uploaded dataset and factored densities");
    return FEM_ERR_STATE;
  }
  FEM_TRY(reset_status(h));
  FEM_TRY(enqueue_estep(h));
  FEM_TRY(sync_status(h));
  if (logl) *logl = h->hstat->logl;
  return FEM_OK;
}

int fem_em_mstep(fem_em *h) {
  FEM_TRY(check_handle(h));
  if (!h->have_post) {
    set_error("M-step needs posteriors (call precompute first)");
    return FEM_ERR_STATE;
  }
  FEM_TRY(reset_status(h));
  FEM_TRY(enqueue_mstep(h));
  h->factored = false;
  return sync_status(h);
}

int fem_em_selftest_wait_expiry(fem_em *h, int64_t budget_cycles, int *roles) {
  FEM_TRY(check_handle(h));
  if (!mixed(h) || !h->tc) {
    set_error("the bounded-wait self-test runs on a mixed-precision handle with d <= 64");
    return FEM_ERR_UNSUPPORTED;
  }
  if (!roles || budget_cycles < 1000 || budget_cycles > 4000000000LL) {
    set_error("self-test budget must be in [1e3, 4e9] cycles");
    return FEM_ERR_BAD_ARG;
  }
  FEM_CUDA(cudaSetDevice(h->cfg.device));
  FEM_TRY(reset_status(h));
  FEM_TRY(em_tc_wait_selftest(h, (long long)budget_cycles, roles));
  h->factored = false;     // TMEM and the status word went through the expiry path
  return sync_status(h);
}

int fem_em_max_condition(fem_em *h, double *cond) {
  FEM_TRY(check_handle(h));
  if (!cond) return FEM_ERR_BAD_ARG;
  return max_cond(h, cond);
}

int fem_em_train(fem_em *h, int svd, double *logl_trace, double *e_trace, int capacity,
                 int *iter_counter, double *logl_out) {
  FEM_TRY(check_handle(h));
  if (!h->have_data || !h->have_params) {
    set_error("train needs an uploaded dataset and parameters");
    return FEM_ERR_STATE;
  }
  FEM_CUDA(cudaSetDevice(h->cfg.device));
  double prev = -DBL_MAX, logl = prev;
  FEM_TRY(reset_status(h));
  FEM_TRY(enqueue_factor(h));
  int st = sync_status(h);
  if (st) {
    h->factored = false;
    return st;
  }
  double cond = 0.0;
  if (svd) {
    FEM_TRY(cond_check(h, &cond));
    if (cond > h->cfg.abort_thr) {
      set_error("Condition number of a covariance matrix is too high (%g)", cond);
      return FEM_ERR_COND_ABORT;
    }
  }
  int it;
  if (h->timing) FEM_CUDA(cudaEventRecord(h->ev[6], h->stream));
  for (it = 1; it <= h->cfg.max_sweeps; it++) {
    FEM_TRY(reset_status(h));
    if (h->timing) h->sweeps++;
    FEM_TRY(enqueue_estep(h));
    FEM_TRY(enqueue_mstep(h));
    FEM_TRY(enqueue_factor(h));
    st = sync_status(h);
    logl = h->hstat->logl;
    if (st) {
      h->factored = false;
      if (iter_counter) *iter_counter = it;
      return st;
    }
    if (svd) {
      FEM_TRY(cond_check(h, &cond));
      if (cond > h->cfg.abort_thr) {
        if (iter_counter) *iter_counter = it;
        set_error("Condition number of a covariance matrix is too high (%g)", cond);
        return FEM_ERR_COND_ABORT;
      }
    }
    double e = std::fabs((logl - prev) / logl);
    if (logl < prev) e = 0.0;
    if (logl_trace && it - 1 < capacity) logl_trace[it - 1] = logl;
    if (e_trace && it - 1 < capacity) e_trace[it - 1] = e;
    prev = logl;
    if (e < h->cfg.eps) {
      it++;
      break;
    }
  }
  if (h->timing) {
    // ev[6] .. ev[7] brackets every sweep of this loop (host waits included)
    FEM_CUDA(cudaEventRecord(h->ev[7], h->stream));
    FEM_CUDA(cudaEventSynchronize(h->ev[7]));
    float ms = 0.f;
    FEM_CUDA(cudaEventElapsedTime(&ms, h->ev[6], h->ev[7]));
    h->t_train += ms;
  }
  if (iter_counter) *iter_counter = it;
  if (logl_out) *logl_out = logl;
  return FEM_OK;
}

int fem_em_get_posteriors(fem_em *h, double *post) {
  FEM_TRY(check_handle(h));
  if (!post || !h->have_post) {
    set_error("no posteriors (run an E-step first)");
    return FEM_ERR_STATE;
  }
  const int64_t chunk = std::max<int64_t>(1, (int64_t)(32u << 20) / h->k);
  double *buf = nullptr;
  FEM_TRY(dalloc(&buf, (size_t)std::min(chunk, h->n) * h->k));
  int st = FEM_OK;
  for (int64_t r0 = 0; r0 < h->n && st == FEM_OK; r0 += chunk) {
    const int64_t rows = std::min(chunk, h->n - r0);
    st = mixed(h) ? em_tc_post_rows(h, r0, rows, buf) : em_post_rows(h, r0, rows, buf);
    if (st == FEM_OK &&
        cudaMemcpyAsync(post + r0 * h->k, buf, (size_t)rows * h->k * sizeof(double),
                        cudaMemcpyDeviceToHost, h->stream) != cudaSuccess)
      st = FEM_ERR_CUDA;
  }
  if (cudaStreamSynchronize(h->stream) != cudaSuccess && st == FEM_OK) st = FEM_ERR_CUDA;
  dfree(buf);
  if (st == FEM_ERR_CUDA) set_error("posterior read-back failed");
  return st;
}

int fem_em_retrieve_classes(fem_em *h, int32_t *classes) {
  FEM_TRY(check_handle(h));
  if (!classes || !h->have_post) {
    set_error("no posteriors (run an E-step first)");
    return FEM_ERR_STATE;
  }
  int32_t *dc = nullptr;
  FEM_TRY(dalloc(&dc, h->n));
  int st = mixed(h) ? em_tc_classes(h, dc) : em_classes(h, dc);
  if (st == FEM_OK &&
      cudaMemcpyAsync(classes, dc, h->n * sizeof(int32_t), cudaMemcpyDeviceToHost, h->stream) != cudaSuccess)
    st = FEM_ERR_CUDA;
  cudaStreamSynchronize(h->stream);
  dfree(dc);
  return st;
}

int fem_em_get_factors(fem_em *h, double *U, double *logdet) {
  FEM_TRY(check_handle(h));
  if (!h->factored) {
    set_error("densities not factored");
    return FEM_ERR_STATE;
  }
  const size_t dd = (size_t)h->d * h->d;
  if (U) {
    std::vector<double> W(dd * h->k);
    FEM_CUDA(cudaMemcpyAsync(W.data(), h->linv, W.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    FEM_CUDA(cudaStreamSynchronize(h->stream));
    // CholInvC = (L^-1)^T
    for (int j = 0; j < h->k; j++)
      for (int r = 0; r < h->d; r++)
        for (int c = 0; c < h->d; c++) U[dd * j + (size_t)r * h->d + c] = W[dd * j + (size_t)c * h->d + r];
  }
  if (logdet)
    FEM_CUDA(cudaMemcpyAsync(logdet, h->logdet, h->k * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  FEM_CUDA(cudaStreamSynchronize(h->stream));
  return FEM_OK;
}

int fem_em_timing_reset(fem_em *h, int enable) {
  FEM_TRY(check_handle(h));
  h->timing = enable != 0;
  h->t_estep = h->t_mstep = h->t_final = h->t_train = h->t_cov = 0.0;
  h->launches = h->sweeps = 0;
  return FEM_OK;
}

int fem_em_timing_total(fem_em *h, double *train_ms, int64_t *sweeps) {
  FEM_TRY(check_handle(h));
  if (train_ms) *train_ms = h->t_train;
  if (sweeps) *sweeps = h->sweeps;
  return FEM_OK;
}

int fem_em_timing_covariance(fem_em *h, double *cov_ms) {
  FEM_TRY(check_handle(h));
  if (cov_ms) *cov_ms = h->t_cov;
  return FEM_OK;
}

int fem_em_timing_get(fem_em *h, double *estep_ms, double *mstep_ms, double *finalize_ms,
                      int64_t *launches) {
  FEM_TRY(check_handle(h));
  if (estep_ms) *estep_ms = h->t_estep;
  if (mstep_ms) *mstep_ms = h->t_mstep;
  if (finalize_ms) *finalize_ms = h->t_final;
  if (launches) *launches = h->launches;
  return FEM_OK;
}

}  // extern "C"
