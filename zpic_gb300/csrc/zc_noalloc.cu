// zc_noalloc.cu -- field energy of caller-owned device grids without any
// device allocation (zc_field_energy_static in include/zpic_cuda.h).
//
// Who needs it: code that computes the energy diagnostic from inside a
// running time loop whose device memory is owned by another allocator -- for
// example a framework whose caching allocator has already reserved the GPU,
// or an embedding that forbids cudaMalloc/cudaFree because they synchronise
// the device and stall the loop.  Such callers hand in the field planes and a
// 6-double output they already own; the per-row partial sums live in the
// fixed array below instead of a per-call allocation.
//
// The array belongs to every GPU that loads this library and stays resident
// until the process exits.  All calls share it and it keeps the contents of
// the last call; every slot a call reads is written earlier in the same call,
// so nothing has to start at zero.  Two calls whose kernels overlap on the
// GPU (different streams, or different threads on one device) race on the
// array and return wrong sums: serialise them.
#include <cstdio>
#include <mutex>

#include "../../include/zpic_cuda.h"
#include "zc_internal.cuh"
#include "zc_kernels.h"

namespace {

// one row of partial sums (6 components) per grid row
static __device__ __align__(256) double g_energy_rows[ZC_STATIC_MAX_ROWS * 6];

// device address of g_energy_rows for each device ordinal, looked up once
// in the runtime's primary context of that device (a cudaDeviceReset in
// the host process makes the cached address stale)
constexpr int kMaxDevices = 64;
double *g_rows_addr[kMaxDevices] = {};
std::mutex g_rows_mutex;

__global__ void __launch_bounds__(256) k_energy_rows(const float *E, const float *B, size_t plane, int pitch,
                                                     int nx, double *rows) {
  __shared__ double sred[8];
  const int by = blockIdx.x + 1;  // buffer row of cell row blockIdx.x
  float s[6] = {0, 0, 0, 0, 0, 0}, c[6] = {0, 0, 0, 0, 0, 0};
  for (int i = threadIdx.x; i < nx; i += blockDim.x) {
    const size_t k = (size_t)by * pitch + i + 1;
#pragma unroll
    for (int q = 0; q < 6; ++q) {
      const float f = (q < 3) ? E[q * plane + k] : B[(q - 3) * plane + k];
      const float y = f * f - c[q];
      const float t = s[q] + y;
      c[q] = (t - s[q]) - y;
      s[q] = t;
    }
  }
  for (int q = 0; q < 6; ++q) {
    const double v = zc::block_sum_double<256>((double)s[q] - (double)c[q], sred);
    if (threadIdx.x == 0) rows[blockIdx.x * 6 + q] = v;
  }
}

__global__ void k_energy_rows_sum(const double *rows, int ny, double *out, float dx, float dy) {
  if (threadIdx.x < 6) {
    double s = 0;
    for (int j = 0; j < ny; ++j) s += rows[j * 6 + threadIdx.x];  // fixed order
    out[threadIdx.x] = s * (0.5 * dx * dy);
  }
}

zc_status reject(zc_status st, const char *msg) {
  zc::set_error_message(msg);
  return st;
}

}  // namespace

extern "C" ZC_API zc_status zc_field_energy_static(const float *E, const float *B, size_t plane, int pitch,
                                                   int nx, int ny, float dx, float dy, double *energy,
                                                   void *stream) {
  char msg[256];
  if (!E || !B || !energy) return reject(ZC_EINVAL, "zc_field_energy_static: null pointer argument");
  if (nx < 1 || ny < 1 || pitch < nx + 3 || plane < (size_t)pitch * (size_t)(ny + 3)) {
    snprintf(msg, sizeof msg, "zc_field_energy_static: inconsistent grid (nx=%d ny=%d pitch=%d plane=%zu)", nx,
             ny, pitch, plane);
    return reject(ZC_EINVAL, msg);
  }
  if (ny > ZC_STATIC_MAX_ROWS) {
    snprintf(msg, sizeof msg,
             "zc_field_energy_static: ny=%d rows exceed the fixed scratch of %d rows (use zc_energy)", ny,
             ZC_STATIC_MAX_ROWS);
    return reject(ZC_EINVAL, msg);
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return reject(ZC_ECUDA, "zc_field_energy_static: no usable current device");
  double *rows = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_rows_mutex);
    if (!g_rows_addr[dev]) {
      // set-up, once per device, with that device current
      cudaError_t e = cudaGetSymbolAddress((void **)&g_rows_addr[dev], g_energy_rows);
      if (e != cudaSuccess) {
        g_rows_addr[dev] = nullptr;
        snprintf(msg, sizeof msg, "zc_field_energy_static: cudaGetSymbolAddress failed: %s",
                 cudaGetErrorString(e));
        return reject(ZC_ECUDA, msg);
      }
    }
    rows = g_rows_addr[dev];
  }
  cudaStream_t st = (cudaStream_t)stream;
  // clear an error left by earlier, unrelated work, so that only this call's
  // launch errors are reported below
  (void)cudaGetLastError();
  k_energy_rows<<<ny, 256, 0, st>>>(E, B, plane, pitch, nx, rows);
  k_energy_rows_sum<<<1, 32, 0, st>>>(rows, ny, energy, dx, dy);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    snprintf(msg, sizeof msg, "zc_field_energy_static: launch failed: %s", cudaGetErrorString(e));
    return reject(ZC_ECUDA, msg);
  }
  return ZC_OK;
}
