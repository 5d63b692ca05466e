// fs_noalloc.cu -- max|div u| of a caller-owned f32 MAC velocity field that
// allocates no device memory.
//
// Who needs this: hosts that own every byte of device memory through their
// own pool (a game engine or a visualisation server that reserves the GPU at
// start-up and forbids later cudaMalloc), and frame loops where cudaMalloc /
// cudaFree are off limits because they can synchronise the whole device and
// stall the frame.  Such a caller passes device pointers it already owns and
// gets the reduction done with scratch the library reserves for itself.
//
// The scratch is the file-scope array g_noalloc_scratch below: one f32 slot
// per 32x8-cell block for the block maxima, then a 32-bit arrival counter.
// Every GPU that loads the library holds it (256 KB) until the process exits.
// Its device address is looked up on the first call on each device and kept;
// after cudaDeviceReset on that device the kept address is stale, so a
// process that resets a device must not call this entry point on it again.
#include <cuda_runtime.h>
#include <math.h>

#include <mutex>
#include <string>

#include "../../include/fluid.h"

namespace fs {
void record_error(const std::string& msg);  // fs_api.cu: message for fs_last_error(NULL)
}

namespace {

constexpr int kBlockX = 32, kBlockY = 8;
// 65536 blocks of 32x8 cells: grids up to 16,777,216 cells (4096 x 4096)
constexpr int kMaxBlocks = 65536;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) float g_noalloc_scratch[kMaxBlocks + 64];

std::mutex g_mu;
float* g_scratch_addr[kMaxDevices];  // device address of g_noalloc_scratch, per device

__device__ __forceinline__ float absnan32(float x) { return x != x ? INFINITY : fabsf(x); }

// (uR - uL)/dx + (vT - vB)/dy per cell (src/core/grid.js:191-206), block
// maxima in scratch[0..nblk), the last block to arrive folds them in a fixed
// order into *out and resets the counter.
__global__ void __launch_bounds__(kBlockX* kBlockY)
    k_maxdiv_noalloc(const float* __restrict__ u, const float* __restrict__ v, int nx, int ny, float idx,
                     float idy, float* __restrict__ scratch, double* __restrict__ out) {
  __shared__ float sm[kBlockX * kBlockY / 32];
  __shared__ bool last;
  const int i = blockIdx.x * kBlockX + threadIdx.x, j = blockIdx.y * kBlockY + threadIdx.y;
  const int tid = threadIdx.y * kBlockX + threadIdx.x, lane = tid & 31, warp = tid >> 5;
  constexpr int nwarp = kBlockX * kBlockY / 32;
  unsigned* counter = reinterpret_cast<unsigned*>(scratch + kMaxBlocks);
  float m = 0.f;
  if (i < nx && j < ny) {
    int ip = i + 1 == nx ? 0 : i + 1, jp = j + 1 == ny ? 0 : j + 1;
    int64_t c = (int64_t)j * nx + i;
    float uL = u[c], uR = u[(int64_t)j * nx + ip], vB = v[c], vT = v[(int64_t)jp * nx + i];
    m = absnan32((uR - uL) * idx + (vT - vB) * idy);
  }
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if (lane == 0) sm[warp] = m;
  __syncthreads();
  const int nblk = gridDim.x * gridDim.y;
  if (tid == 0) {
    float t = sm[0];
    for (int w = 1; w < nwarp; w++) t = fmaxf(t, sm[w]);
    scratch[blockIdx.y * gridDim.x + blockIdx.x] = t;
    __threadfence();
    last = atomicAdd(counter, 1u) == (unsigned)nblk - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  float t = 0.f;
  for (int k = tid; k < nblk; k += kBlockX * kBlockY) t = fmaxf(t, ((volatile float*)scratch)[k]);
  for (int o = 16; o > 0; o >>= 1) t = fmaxf(t, __shfl_xor_sync(0xffffffffu, t, o));
  __syncthreads();
  if (lane == 0) sm[warp] = t;
  __syncthreads();
  if (tid == 0) {
    float f = sm[0];
    for (int w = 1; w < nwarp; w++) f = fmaxf(f, sm[w]);
    *out = (double)f;
    *counter = 0u;
  }
}

int fail(int code, const std::string& msg) {
  fs::record_error(msg);
  return code;
}

}  // namespace

extern "C" FS_API int fs_max_divergence_noalloc(const float* d_u, const float* d_v, int32_t nx, int32_t ny,
                                                double lx, double ly, double* d_out, void* stream) {
  if (!d_u || !d_v || !d_out) return fail(FS_ERR_INVALID_ARGUMENT, "fs_max_divergence_noalloc: NULL pointer");
  if (nx < 2 || ny < 2 || !(lx > 0) || !(ly > 0))
    return fail(FS_ERR_INVALID_ARGUMENT, "fs_max_divergence_noalloc: grid must be >= 2x2 with a positive domain");
  const int gx = (nx + kBlockX - 1) / kBlockX, gy = (ny + kBlockY - 1) / kBlockY;
  if (gy > 65535)  // the launch's grid-y limit (a narrow, very tall grid)
    return fail(FS_ERR_INVALID_ARGUMENT,
                "fs_max_divergence_noalloc: ny = " + std::to_string(ny) +
                    " needs more than 65535 rows of 32x8-cell blocks; the static scratch kernel takes "
                    "ny <= 524280");
  if ((int64_t)gx * gy > kMaxBlocks)
    return fail(FS_ERR_INVALID_ARGUMENT,
                "fs_max_divergence_noalloc: grid needs " + std::to_string((int64_t)gx * gy) +
                    " blocks of 32x8 cells; the static scratch holds 65536 (at most 16,777,216 cells, "
                    "e.g. 4096 x 4096)");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(FS_ERR_NO_DEVICE, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return fail(FS_ERR_UNSUPPORTED, "device ordinal above 63");
  float* scratch;
  {
    // first call on this device: resolve the device address of the static
    // array with that device current (the array's name is only a host-side
    // stand-in in host code)
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_addr[dev]) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess)
        return fail(FS_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      g_scratch_addr[dev] = static_cast<float*>(p);
    }
    scratch = g_scratch_addr[dev];
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // the arrival counter must start at zero (the previous call reset it, but a
  // call that failed mid-way would not have)
  e = cudaMemsetAsync(scratch + kMaxBlocks, 0, sizeof(unsigned), st);
  if (e != cudaSuccess) return fail(FS_ERR_CUDA, std::string("cudaMemsetAsync: ") + cudaGetErrorString(e));
  const float idx = (float)(1.0 / (lx / nx)), idy = (float)(1.0 / (ly / ny));
  k_maxdiv_noalloc<<<dim3(gx, gy), dim3(kBlockX, kBlockY), 0, st>>>(d_u, d_v, nx, ny, idx, idy, scratch, d_out);
  e = cudaGetLastError();
  if (e != cudaSuccess) return fail(FS_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
  return FS_OK;
}
