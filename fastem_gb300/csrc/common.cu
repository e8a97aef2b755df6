// common.cu -- error reporting, device selection and host-side helpers.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <map>
#include <mutex>
#include <utility>
#include <vector>

#include "fem_internal.cuh"

namespace fem {

static thread_local char g_err[512] = "";

void set_error(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

static std::mutex g_smem_mu;
static std::map<std::pair<const void *, int>, int> g_smem_limit;

cudaError_t allow_dyn_smem(const void *func, size_t bytes) {
  if (bytes <= 48 * 1024) return cudaSuccess;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lock(g_smem_mu);
  int &cur = g_smem_limit[{func, dev}];
  if ((int)bytes <= cur) return cudaSuccess;
  e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e == cudaSuccess) cur = (int)bytes;
  return e;
}

static int g_sms = 0;

int sm_count() { return g_sms > 0 ? g_sms : kSMs; }

int select_device(int device) {
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0) {
    set_error("no CUDA device: %s", e != cudaSuccess ? cudaGetErrorString(e) : "count is 0");
    return FEM_ERR_NO_DEVICE;
  }
  if (device < 0 || device >= count) {
    set_error("device %d out of range (%d devices)", device, count);
    return FEM_ERR_BAD_ARG;
  }
  cudaDeviceProp p;
  FEM_CUDA(cudaGetDeviceProperties(&p, device));
  if (p.major != 10 || p.minor != 3) {
    set_error("device %d is sm_%d%d; this library is built for sm_103a only", device, p.major,
              p.minor);
    return FEM_ERR_NO_DEVICE;
  }
  FEM_CUDA(cudaSetDevice(device));
  g_sms = p.multiProcessorCount;
  return FEM_OK;
}

// cuTensorMapEncodeTiled resolved through the runtime, so the library does
// not link libcuda (it must load on hosts without a driver).
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *,
                                  CUtensorMapInterleave, CUtensorMapSwizzle, CUtensorMapL2promotion,
                                  CUtensorMapFloatOOBfill);

int encode_tmap_2d(CUtensorMap *m, CUtensorMapDataType dt, int elem_bytes, const void *base, uint64_t cols,
                   uint64_t rows, uint32_t box_cols, uint32_t box_rows, CUtensorMapSwizzle swz,
                   uint64_t pitch_bytes) {
  static EncodeTiledFn fn = nullptr;
  if (!fn) {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !p) {
      set_error("cuTensorMapEncodeTiled is not available from the driver");
      return FEM_ERR_CUDA;
    }
    fn = (EncodeTiledFn)p;
  }
  cuuint64_t dims[2] = {cols, rows};
  cuuint64_t strides[1] = {pitch_bytes ? pitch_bytes : cols * (uint64_t)elem_bytes};
  cuuint32_t box[2] = {box_cols, box_rows};
  cuuint32_t es[2] = {1, 1};
  CUresult r = fn(m, dt, 2, const_cast<void *>(base), dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, swz,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled failed (CUresult %d)", (int)r);
    return FEM_ERR_CUDA;
  }
  return FEM_OK;
}

}  // namespace fem

extern "C" int fem_api_version(void) { return FEM_API_VERSION; }

extern "C" const char *fem_last_error(void) { return fem::g_err; }
