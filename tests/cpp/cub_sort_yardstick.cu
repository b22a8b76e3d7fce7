// Yardstick for the onesweep sort (a measurement only, never a code path of
// the library): times the CUDA toolkit's own radix sort,
// cub::DeviceRadixSort::SortPairs (or SortKeys) on n uint32 keys (hashed,
// uniform 32-bit) with uint32 iota values, 10 timed sorts after 3 warm-up
// sorts, CUDA events around each sort, fresh keys before each, and prints one
// JSON line.  Usage: cub_sort_yardstick [n] [keys_only]
#include <cub/cub.cuh>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>

#define CK(x)                                                                        \
  do {                                                                               \
    cudaError_t e = (x);                                                             \
    if (e != cudaSuccess) {                                                          \
      std::printf("CUDA %s at %d\n", cudaGetErrorString(e), __LINE__);               \
      return 1;                                                                      \
    }                                                                                \
  } while (0)

__global__ void fill(uint32_t *k, uint32_t *v, size_t n, uint64_t seed) {
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) {
    uint64_t x = (i + seed) * 0x9E3779B97F4A7C15ull;
    x ^= x >> 31;
    x *= 0xBF58476D1CE4E5B9ull;
    x ^= x >> 29;
    k[i] = uint32_t(x >> 16);
    v[i] = uint32_t(i);
  }
}

int main(int argc, char **argv) {
  const size_t n = argc > 1 ? std::strtoull(argv[1], nullptr, 0) : (size_t(1) << 28);
  const int keys_only = argc > 2 ? std::atoi(argv[2]) : 0;
  uint32_t *k0, *k1, *v0, *v1;
  CK(cudaMalloc(&k0, n * 4));
  CK(cudaMalloc(&k1, n * 4));
  CK(cudaMalloc(&v0, n * 4));
  CK(cudaMalloc(&v1, n * 4));
  size_t tb = 0;
  void *tmp = nullptr;
  cub::DoubleBuffer<uint32_t> dk(k0, k1), dv(v0, v1);
  if (keys_only) CK(cub::DeviceRadixSort::SortKeys(nullptr, tb, dk, n));
  else CK(cub::DeviceRadixSort::SortPairs(nullptr, tb, dk, dv, n));
  CK(cudaMalloc(&tmp, tb));
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  std::vector<float> ms;
  for (int it = 0; it < 13; ++it) {
    fill<<<1216, 256>>>(dk.Current(), dv.Current(), n, uint64_t(it) * 977);
    CK(cudaDeviceSynchronize());
    cudaEventRecord(a);
    if (keys_only) cub::DeviceRadixSort::SortKeys(tmp, tb, dk, n);
    else cub::DeviceRadixSort::SortPairs(tmp, tb, dk, dv, n);
    cudaEventRecord(b);
    CK(cudaEventSynchronize(b));
    float t = 0.f;
    cudaEventElapsedTime(&t, a, b);
    if (it >= 3) ms.push_back(t);
  }
  std::vector<uint32_t> h(n);
  CK(cudaMemcpy(h.data(), dk.Current(), n * 4, cudaMemcpyDeviceToHost));
  size_t bad = 0;
  for (size_t i = 1; i < n; ++i) bad += h[i] < h[i - 1];
  double sum = 0, mn = 1e9;
  for (float t : ms) {
    sum += t;
    if (t < mn) mn = t;
  }
  const double mean = sum / ms.size();
  std::printf("{\"yardstick\": \"cub::DeviceRadixSort::%s uint32%s\", \"n\": %zu, \"ms_mean\": %.4f, "
              "\"ms_min\": %.4f, \"gkeys_s\": %.3f, \"unsorted\": %zu}\n",
              keys_only ? "SortKeys" : "SortPairs", keys_only ? "" : "/uint32", n, mean, mn, n / mean / 1e6, bad);
  return bad ? 1 : 0;
}
