/*
 * p2m_noalloc.cu -- p2m_map_sums_noalloc: the sums of up to P2M_NOALLOC_MAXMAPS float maps
 * already in device memory, computed without allocating anything.
 *
 * The kernel is the map-sum reduction of the statistics read-out (float-float partial
 * sums per thread, FP64 per-thread totals added atomically), writing into a file-scope
 * device array instead of a context's scratch.  The host side makes no cudaMalloc,
 * cudaFree or other allocating call: it looks the array's address up once per device
 * (cudaGetSymbolAddress, with that device current), clears it, launches, and copies the
 * sums back.
 *
 * Contract:
 *  - the scratch array is per device and shared by every call on that device: calls that
 *    overlap in time on one device (two host threads, or two streams) race on it and
 *    must be serialised by the caller;
 *  - the scratch must start at zero for each call; the call clears it itself, on the
 *    caller's stream, before the launch;
 *  - the first call on a device does the one-time set-up (the symbol lookup, which can
 *    load the module): make it before any stream capture begins;
 *  - the looked-up address belongs to the device's current context: after a
 *    cudaDeviceReset (by this process or a host framework) it is stale and later calls
 *    would write through a freed address, so the call must not be used across a reset;
 *  - the call is synchronous: it returns after the sums have reached the host, which a
 *    stream under capture cannot do, so a capturing stream is refused with
 *    P2M_ERR_STATE before anything is queued;
 *  - more than P2M_NOALLOC_MAXMAPS maps is rejected with P2M_ERR_CAPACITY.
 */
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/p2m.h"
#include "../../include/p2m_tools.h"

#define FULL_MASK 0xffffffffu
#define P2M_NOALLOC_MAX_DEVICES 64

/* the statically sized scratch: one FP64 total per map (64 bytes) */
static __device__ __align__(256) double g_noalloc_sums[P2M_NOALLOC_MAXMAPS];

struct NoallocMaps {
  const float *p[P2M_NOALLOC_MAXMAPS];
};

/* blockIdx.y selects the map; each thread keeps a float-float (TwoSum) partial sum */
__global__ void __launch_bounds__(256) k_map_sums_static(NoallocMaps maps, long long n) {
  const float *map = maps.p[blockIdx.y];
  float hi = 0.0f, lo = 0.0f;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < n;
       p += (long long)gridDim.x * blockDim.x) {
    const float x = map[p];
    const float sm = __fadd_rn(hi, x);
    const float bb = __fsub_rn(sm, hi);
    lo = __fadd_rn(lo, __fadd_rn(__fsub_rn(hi, __fsub_rn(sm, bb)), __fsub_rn(x, bb)));
    hi = sm;
  }
  double s = (double)hi + (double)lo;
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(FULL_MASK, s, o);
  if ((threadIdx.x & 31) == 0 && s != 0.0) atomicAdd(&g_noalloc_sums[blockIdx.y], s);
}

namespace {

std::mutex g_setup_mutex;
double *g_scratch[P2M_NOALLOC_MAX_DEVICES] = {};
int g_nsm[P2M_NOALLOC_MAX_DEVICES] = {};

/* address of this device's scratch and its SM count, looked up once per device with the
   device current */
cudaError_t device_scratch(int dev, double **scratch, int *nsm) {
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch[dev]) {
    void *addr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&addr, g_noalloc_sums);
    if (e != cudaSuccess) return e;
    int sms = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    g_nsm[dev] = sms;
    g_scratch[dev] = (double *)addr;
  }
  *scratch = g_scratch[dev];
  *nsm = g_nsm[dev];
  return cudaSuccess;
}

}  // namespace

extern "C" p2m_status p2m_map_sums_noalloc(const float *const *d_maps, int32_t nmaps,
                                           int64_t npix, double *sums, void *stream) {
  if (!d_maps || !sums || nmaps < 1 || npix < 0) return P2M_ERR_BADARG;
  if (nmaps > P2M_NOALLOC_MAXMAPS) return P2M_ERR_CAPACITY;
  NoallocMaps maps = {};
  for (int m = 0; m < nmaps; m++) {
    if (!d_maps[m] && npix > 0) return P2M_ERR_BADARG;
    maps.p[m] = d_maps[m];
  }
  cudaStreamCaptureStatus cap_st = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing((cudaStream_t)stream, &cap_st) != cudaSuccess) return P2M_ERR_CUDA;
  if (cap_st != cudaStreamCaptureStatusNone) return P2M_ERR_STATE;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return P2M_ERR_CUDA;
  if (dev < 0 || dev >= P2M_NOALLOC_MAX_DEVICES) return P2M_ERR_CAPACITY;
  double *scratch = nullptr;
  int nsm = 0;
  if (device_scratch(dev, &scratch, &nsm) != cudaSuccess) return P2M_ERR_CUDA;
  cudaStream_t s = (cudaStream_t)stream;
  const size_t bytes = sizeof(double) * (size_t)nmaps;
  if (cudaMemsetAsync(scratch, 0, bytes, s) != cudaSuccess) return P2M_ERR_CUDA;
  if (npix > 0) {
    /* the statistics read-out's grid (at most 8 blocks per SM): the same per-thread
       partial sums, so the totals differ only by the order of the FP64 atomic adds */
    long long blocks = (npix + 255) / 256;
    long long cap = 8LL * (nsm > 0 ? nsm : 1);
    dim3 grid((unsigned)(blocks < cap ? blocks : cap), (unsigned)nmaps);
    k_map_sums_static<<<grid, 256, 0, s>>>(maps, (long long)npix);
    if (cudaGetLastError() != cudaSuccess) return P2M_ERR_CUDA;
  }
  if (cudaMemcpyAsync(sums, scratch, bytes, cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return P2M_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return P2M_ERR_CUDA;
  return P2M_OK;
}
