// order.cu - spatial order of the stations for the kernels that give each
// thread one station.
//
// A warp decides per column, by vote, whether the column lies in some lane's
// near box and whether every lane is far enough for the second-order form.
// Stations given in an arbitrary order put distant stations in one warp, so
// most columns take the slower branch for the whole warp; the blocks of a
// persistent grid then also wait on one another at the stage barriers.  A
// Z-order (Morton) sort of the stations' home cells keeps the 32 lanes of a
// warp on a compact patch.  The permutation only decides which thread
// computes which station: every station's sum is written at its own index,
// so the result does not depend on it beyond the float grouping.
#include <cub/device/device_radix_sort.cuh>

#include <algorithm>

#include "ztm_internal.cuh"

namespace {

__device__ __forceinline__ uint32_t spread16(uint32_t v) {
  v &= 0xffffu;
  v = (v | (v << 8)) & 0x00ff00ffu;
  v = (v | (v << 4)) & 0x0f0f0f0fu;
  v = (v | (v << 2)) & 0x33333333u;
  v = (v | (v << 1)) & 0x55555555u;
  return v;
}

// key = interleaved bits of the home cell (x, y), clamped to 16 bits each
// (si: the home cell's x, y as the first two of `stride` ints per station;
// cells outside the mesh sort with the nearest edge cell)
__global__ void station_key_kernel(int ns, const int* __restrict__ si, int stride, int nx, int ny,
                                   uint32_t* __restrict__ key, int* __restrict__ idx) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= ns) return;
  const uint32_t x = (uint32_t)min(max(si[(size_t)s * stride], 0), nx - 1);
  const uint32_t y = (uint32_t)min(max(si[(size_t)s * stride + 1], 0), ny - 1);
  key[s] = spread16(x) | (spread16(y) << 1);
  idx[s] = s;
}

// key bits: 2 x the bits of the larger clamped cell index
int key_bits(int nx, int ny) {
  const int n = std::min(std::max(std::max(nx, ny), 2), 65536) - 1;
  int b = 0;
  while ((1 << b) <= n) b++;
  return 2 * b;
}

size_t sort_temp_bytes(int ns, int bits) {
  size_t b = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, b, (const uint32_t*)nullptr, (uint32_t*)nullptr,
                                  (const int*)nullptr, (int*)nullptr, ns, 0, bits,
                                  (cudaStream_t)0);
  return b;
}

}  // namespace

size_t ztm_station_order_ws(int ns, int nx, int ny) {
  if (ns <= 0) return 0;
  return 3 * WsCarver::need((size_t)ns * 4) + WsCarver::need(sort_temp_bytes(ns, key_bits(nx, ny)));
}

int ztm_station_order(ztm_ctx* c, cudaStream_t stream, int ns, const int* si, int stride, int nx,
                      int ny, int* perm, WsCarver& wc) {
  if (ns <= 0) return 0;
  nx = std::min(std::max(nx, 1), 65536);
  ny = std::min(std::max(ny, 1), 65536);
  const int bits = key_bits(nx, ny);
  uint32_t* key = wc.take<uint32_t>(ns);
  uint32_t* key_sorted = wc.take<uint32_t>(ns);
  int* idx = wc.take<int>(ns);
  size_t tb = sort_temp_bytes(ns, bits);
  void* tmp = wc.take<char>(tb);
  station_key_kernel<<<(ns + 255) / 256, 256, 0, stream>>>(ns, si, stride, nx, ny, key, idx);
  c->launches++;
  // a library sort (its kernels are not counted as this library's launches)
  cudaError_t e = cub::DeviceRadixSort::SortPairs(tmp, tb, key, key_sorted, idx, perm, ns, 0, bits,
                                                  stream);
  return ztm_cuda_check(c, e, "station order sort");
}
