// Exact two-material Riemann solves without any device allocation.
//
// Some callers cannot allocate device memory: a host application that owns a
// fixed device-memory budget and hands the library only its own buffers, code
// running while another component forbids new allocations, or a plugin loaded
// into a process whose allocator must not be bypassed.  For them this file
// provides m2cg_riemann_batch_noalloc: the same solver as m2cg_riemann_batch,
// with its only scratch -- the integration-path cache of the adaptive
// rarefaction integration -- in a file-scope device array instead of a
// cudaMalloc'ed buffer.  The caller passes device pointers for every input and
// output; nothing here calls cudaMalloc, cudaFree or an allocating library
// routine.
//
// The array is M2CG_NOALLOC_SCRATCH_BYTES (32 MiB) and lives on every GPU that
// loads the library until the process exits.  All calls share it and it keeps
// the last call's contents; nothing in it has to start at zero (each solve
// writes every cache entry before it reads it).  Calls that overlap on one GPU,
// for example on two streams, race on the array: serialize them.  The first
// call on a device looks up the array's device address; make that first call
// before any stream capture.  A device reset (cudaDeviceReset) ends the
// context the address belongs to; the next call notices the new context and
// looks the address up again.
//
// Compiled without floating-point contraction, like the other interface kernels,
// so its results equal m2cg_riemann_batch's for the same path-cache capacity.
#include <mutex>
#include "m2cg_internal.h"

#define M2CG_NOALLOC_SCRATCH_BYTES (32ull << 20)
#define M2CG_NOALLOC_MAX_PATH_CAP 1024
#define M2CG_NOALLOC_MAX_DEVICES 64

static __device__ __align__(256) double g_noalloc_scratch[M2CG_NOALLOC_SCRATCH_BYTES / sizeof(double)];

m2cg_status m2cg_fill_params(const m2cg_config& c, m2cg::Params& P);
void m2cg_set_error(const char* fmt, ...);

namespace m2cg {

// One thread per problem (grid-stride); the materials are staged in shared memory.
__global__ void __launch_bounds__(128) k_riemann_batch_noalloc(
    Mats mats, RiemannPrm rp, int n_mat, int64_t n, const double* __restrict__ Vm, const int32_t* __restrict__ idm,
    const double* __restrict__ Vp, const int32_t* __restrict__ idp, const double* __restrict__ dir, double* Vs,
    int32_t* id, double* Vsm, double* Vsp, int32_t* iters, int32_t* err, double* scratch, int path_cap) {
  __shared__ Mats sm;
  const int words = (int)(sizeof(Mats) / sizeof(int));
  for (int w = threadIdx.x; w < words; w += blockDim.x) reinterpret_cast<int*>(&sm)[w] = reinterpret_cast<const int*>(&mats)[w];
  __syncthreads();
  int64_t T = (int64_t)gridDim.x * blockDim.x;
  int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  ExactRiemannDev rs;
  rs.mats = &sm;
  rs.P = rp;
  rs.warm_p = 0.0;
  rs.path1.base = scratch + tid;
  rs.path1.stride = T;
  rs.path1.cap = path_cap;
  rs.path3.base = scratch + (int64_t)3 * path_cap * T + tid;
  rs.path3.stride = T;
  rs.path3.cap = path_cap;
  for (int64_t q = tid; q < n; q += T) {
    int a = idm[q], b = idp[q];
    if (a < 0 || a >= n_mat || b < 0 || b >= n_mat) {   // invalid material ID: no solve
      if (err) err[q] = -2;
      if (iters) iters[q] = 0;
      id[q] = -1;
      const double nan = __longlong_as_double(0x7ff8000000000000ll);
      for (int p = 0; p < 5; p++) { Vs[q * 5 + p] = nan; Vsm[q * 5 + p] = nan; Vsp[q * 5 + p] = nan; }
      continue;
    }
    int oid = 0;
    int e = rs.solve(&dir[q * 3], &Vm[q * 5], a, &Vp[q * 5], b, &Vs[q * 5], oid, &Vsm[q * 5], &Vsp[q * 5]);
    id[q] = oid;
    if (iters) iters[q] = rs.evals;
    if (err) err[q] = e;
  }
}

}  // namespace m2cg

using namespace m2cg;

static std::mutex g_noalloc_mutex;
static double* g_noalloc_ptr[M2CG_NOALLOC_MAX_DEVICES];
// the context the cached address belongs to: a device reset destroys the
// primary context, and the array's address must be looked up again in the new
// one (context IDs are unique within a process, handles may be reused)
static unsigned long long g_noalloc_ctx[M2CG_NOALLOC_MAX_DEVICES];

typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long*);

// ID of the calling thread's current context, or 0 when the driver cannot tell.
static unsigned long long current_context_id() {
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  if (!get_current || !get_id) {
    void* f = nullptr;
    void* g = nullptr;
    cudaDriverEntryPointQueryResult q1, q2;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 4000, cudaEnableDefault, &q1) != cudaSuccess ||
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &g, 12000, cudaEnableDefault, &q2) != cudaSuccess ||
        q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f || !g) {
      cudaGetLastError();
      return 0;
    }
    get_current = (CtxGetCurrentFn)f;
    get_id = (CtxGetIdFn)g;
  }
  CUcontext c = nullptr;
  unsigned long long idv = 0;
  if (get_current(&c) != CUDA_SUCCESS || !c || get_id(c, &idv) != CUDA_SUCCESS) return 0;
  return idv;
}

extern "C" m2cg_status m2cg_riemann_batch_noalloc(const m2cg_config* cfg, int64_t n, const double* Vm,
                                                  const int32_t* idm, const double* Vp, const int32_t* idp,
                                                  const double* dir, double* Vs, int32_t* id, double* Vsm,
                                                  double* Vsp, int32_t* iters, int32_t* err, int32_t path_cap,
                                                  void* stream) {
  if (!cfg || n < 0) { m2cg_set_error("null config or negative size"); return M2CG_ERR_INVALID_ARG; }
  if (n == 0) return M2CG_OK;
  if (!Vm || !idm || !Vp || !idp || !dir || !Vs || !id || !Vsm || !Vsp) {
    m2cg_set_error("null device pointer");
    return M2CG_ERR_INVALID_ARG;
  }
  if (path_cap < 2 || path_cap > M2CG_NOALLOC_MAX_PATH_CAP) {
    m2cg_set_error("path_cap %d outside [2, %d]: the static scratch (%llu MiB) holds at most %d cache entries per wave",
                   path_cap, M2CG_NOALLOC_MAX_PATH_CAP, M2CG_NOALLOC_SCRATCH_BYTES >> 20, M2CG_NOALLOC_MAX_PATH_CAP);
    return M2CG_ERR_CAPACITY;
  }
  Params P;
  m2cg_status st = m2cg_fill_params(*cfg, P);
  if (st != M2CG_OK) return st;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= M2CG_NOALLOC_MAX_DEVICES) {
    m2cg_set_error("cudaGetDevice failed or device index %d unsupported", dev);
    return M2CG_ERR_CUDA;
  }
  // make the device's primary context current (created here if the process
  // has not used the device yet), so that the lookup below runs in it
  e = cudaSetDevice(dev);
  if (e != cudaSuccess) {
    m2cg_set_error("cudaSetDevice(%d) failed: %s", dev, cudaGetErrorString(e));
    return M2CG_ERR_CUDA;
  }
  const unsigned long long ctx_id = current_context_id();
  double* scratch;
  {
    // first call on this device (or in a new context after a device reset):
    // host code cannot use the array's name as a device address, so fetch the
    // address once with the device current
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[dev] || g_noalloc_ctx[dev] != ctx_id) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess || !p) {
        m2cg_set_error("cudaGetSymbolAddress(scratch) failed: %s", cudaGetErrorString(e));
        return M2CG_ERR_CUDA;
      }
      g_noalloc_ptr[dev] = (double*)p;
      g_noalloc_ctx[dev] = ctx_id;
    }
    scratch = g_noalloc_ptr[dev];
  }
  // concurrency from the scratch size: 6 * path_cap doubles per solver thread
  int64_t threads = (int64_t)(M2CG_NOALLOC_SCRATCH_BYTES / sizeof(double)) / (6ll * path_cap);
  threads = (threads / 128) * 128;
  int blocks = (int)(threads / 128);
  k_riemann_batch_noalloc<<<blocks, 128, 0, (cudaStream_t)stream>>>(P.mats, P.rp, P.n_mat, n, Vm, idm, Vp, idp, dir,
                                                                     Vs, id, Vsm, Vsp, iters, err, scratch, path_cap);
  e = cudaGetLastError();
  if (e != cudaSuccess) {
    m2cg_set_error("kernel launch failed: %s", cudaGetErrorString(e));
    return M2CG_ERR_CUDA;
  }
  return M2CG_OK;
}
