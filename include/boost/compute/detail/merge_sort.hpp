// boost/compute/detail/merge_sort.hpp -- stable sort with a user comparator.
//
// Reference: sort(first, last, compare) with a comparator the radix path does
// not cover (a lambda, a BOOST_COMPUTE_FUNCTION) runs merge_sort_on_gpu
// (detail/merge_sort_on_gpu.hpp:32-590): a block sort then merge passes.
// Here the comparator is compiled (NVRTC, program cache) into three kernels:
//   bcx_ms_block  -- each 256-thread block sorts a 1024-element tile: every
//                    thread insertion-sorts its 4 elements in registers, then
//                    runs of 4, 8, ..., 512 are merged in shared memory, each
//                    thread finding its place on the merge path by binary
//                    search and emitting 4 outputs;
//   bcx_ms_merge  -- one pass merges runs of width w into runs of 2w in global
//                    memory, every thread locating its 4 outputs on the merge
//                    path of its run pair the same way;
//   passes ping-pong between the caller's buffers and a temporary, and a final
//   copy returns the result if it ended in the temporary.
// Ties take the left run first at every level, so the sort is stable (as
// stable_sort requires); values, when present, move with their keys.
#ifndef BOOST_COMPUTE_DETAIL_MERGE_SORT_HPP
#define BOOST_COMPUTE_DETAIL_MERGE_SORT_HPP

#include <sstream>
#include <string>
#include <utility>

#include <boost/compute/container/vector.hpp>
#include <boost/compute/detail/jit.hpp>

namespace boost {
namespace compute {
namespace detail {

constexpr unsigned kMergeThreads = 256;
constexpr unsigned kMergeItems = 4;
constexpr unsigned kMergeTile = kMergeThreads * kMergeItems;

inline std::string merge_sort_source(const std::string &defs, const std::string &less_expr, const char *kt,
                                     const char *vt) {
  const bool has_v = vt != nullptr;
  std::ostringstream s;
  s << jit_prelude() << defs << "\n"
    << "typedef " << kt << " K;\n"
    << "typedef " << (has_v ? vt : "unsigned char") << " V;\n"
    << "#define HAS_V " << (has_v ? 1 : 0) << "\n"
    << "#define THREADS " << kMergeThreads << "\n#define IPT " << kMergeItems << "\n#define TILE " << kMergeTile
    << "\n"
    << "__device__ __forceinline__ bool bcx_less(const K &_1, const K &_2) { return (" << less_expr << "); }\n"
    // number of elements taken from A among the first o outputs of the stable
    // merge of A (length na) and B (length nb)
    << "template <class PA, class PB>\n"
    << "__device__ __forceinline__ unsigned long long merge_path(PA A, unsigned long long na, PB B,"
       " unsigned long long nb, unsigned long long o) {\n"
    << "  unsigned long long lo = o > nb ? o - nb : 0, hi = o < na ? o : na;\n"
    << "  while (lo < hi) {\n"
    << "    const unsigned long long mid = (lo + hi) / 2;\n"
    << "    if (!bcx_less(B[o - mid - 1], A[mid])) lo = mid + 1; else hi = mid;\n"
    << "  }\n"
    << "  return lo;\n"
    << "}\n"
    << "extern \"C\" __global__ void __launch_bounds__(THREADS) bcx_ms_block(K *keys, V *vals,"
       " unsigned long long n) {\n"
    << "  __shared__ K sk[2][TILE];\n"
    << "#if HAS_V\n  __shared__ V sv[2][TILE];\n#endif\n"
    << "  const unsigned long long base = (unsigned long long)blockIdx.x * TILE;\n"
    << "  const unsigned m = (unsigned)(n - base < TILE ? n - base : TILE);\n"
    << "  for (unsigned i = threadIdx.x; i < m; i += THREADS) {\n"
    << "    sk[0][i] = keys[base + i];\n"
    << "#if HAS_V\n    sv[0][i] = vals[base + i];\n#endif\n  }\n"
    << "  __syncthreads();\n"
    // registers: stable insertion sort of this thread's IPT elements
    << "  const unsigned t0 = threadIdx.x * IPT;\n"
    << "  const unsigned cnt = t0 < m ? (m - t0 < IPT ? m - t0 : IPT) : 0;\n"
    << "  K rk[IPT];\n#if HAS_V\n  V rv[IPT];\n#endif\n"
    << "  for (unsigned i = 0; i < cnt; ++i) {\n"
    << "    K k = sk[0][t0 + i];\n#if HAS_V\n    V v = sv[0][t0 + i];\n#endif\n"
    << "    unsigned j = i;\n"
    << "    while (j > 0 && bcx_less(k, rk[j - 1])) {\n"
    << "      rk[j] = rk[j - 1];\n#if HAS_V\n      rv[j] = rv[j - 1];\n#endif\n      --j;\n    }\n"
    << "    rk[j] = k;\n#if HAS_V\n    rv[j] = v;\n#endif\n  }\n"
    << "  __syncthreads();\n"
    << "  for (unsigned i = 0; i < cnt; ++i) {\n"
    << "    sk[0][t0 + i] = rk[i];\n#if HAS_V\n    sv[0][t0 + i] = rv[i];\n#endif\n  }\n"
    << "  __syncthreads();\n"
    << "  int cur = 0;\n"
    << "  for (unsigned w = IPT; w < m; w *= 2) {\n"
    << "    if (t0 < m) {\n"
    << "      const unsigned p0 = (t0 / (2 * w)) * (2 * w);\n"
    << "      const unsigned a0 = p0, a1 = p0 + w < m ? p0 + w : m, b1 = p0 + 2 * w < m ? p0 + 2 * w : m;\n"
    << "      const K *A = &sk[cur][a0];\n      const K *B = &sk[cur][a1];\n"
    << "      const unsigned na = a1 - a0, nb = b1 - a1, o = t0 - p0;\n"
    << "      unsigned i = (unsigned)merge_path(A, na, B, nb, o), j = o - i;\n"
    << "      for (unsigned q = 0; q < IPT && t0 + q < m; ++q) {\n"
    << "        const bool take_a = i < na && (j >= nb || !bcx_less(B[j], A[i]));\n"
    << "        const unsigned src = take_a ? a0 + i : a1 + j;\n"
    << "        sk[cur ^ 1][t0 + q] = sk[cur][src];\n"
    << "#if HAS_V\n        sv[cur ^ 1][t0 + q] = sv[cur][src];\n#endif\n"
    << "        if (take_a) ++i; else ++j;\n"
    << "      }\n"
    << "    }\n"
    << "    cur ^= 1;\n"
    << "    __syncthreads();\n"
    << "  }\n"
    << "  for (unsigned i = threadIdx.x; i < m; i += THREADS) {\n"
    << "    keys[base + i] = sk[cur][i];\n#if HAS_V\n    vals[base + i] = sv[cur][i];\n#endif\n  }\n"
    << "}\n"
    << "extern \"C\" __global__ void __launch_bounds__(THREADS) bcx_ms_merge(const K *__restrict__ ik,"
       " const V *__restrict__ iv, K *__restrict__ ok, V *__restrict__ ov, unsigned long long n,"
       " unsigned long long w) {\n"
    << "  const unsigned long long g = ((unsigned long long)blockIdx.x * THREADS + threadIdx.x) * IPT;\n"
    << "  if (g >= n) return;\n"
    << "  const unsigned long long p0 = (g / (2 * w)) * (2 * w);\n"
    << "  const unsigned long long a1 = p0 + w < n ? p0 + w : n, b1 = p0 + 2 * w < n ? p0 + 2 * w : n;\n"
    << "  const unsigned long long na = a1 - p0, nb = b1 - a1, o = g - p0;\n"
    << "  const K *A = ik + p0;\n  const K *B = ik + a1;\n"
    << "  unsigned long long i = merge_path(A, na, B, nb, o), j = o - i;\n"
    << "  for (unsigned q = 0; q < IPT && g + q < n; ++q) {\n"
    << "    const bool take_a = i < na && (j >= nb || !bcx_less(B[j], A[i]));\n"
    << "    const unsigned long long src = take_a ? p0 + i : a1 + j;\n"
    << "    ok[g + q] = ik[src];\n#if HAS_V\n    ov[g + q] = iv[src];\n#endif\n"
    << "    if (take_a) ++i; else ++j;\n"
    << "  }\n"
    << "}\n";
  return s.str();
}

// Stable sort of keys[0, n) (and values, when vals != nullptr) by the
// kernel-side expression less_expr of (_1, _2).
template <class K, class V>
inline void jit_merge_sort(K *keys, V *vals, size_t n, const std::string &defs, const std::string &less_expr,
                           command_queue &queue) {
  if (n < 2) return;
  const char *vt = vals ? cuda_type_name<V>::get() : nullptr;
  const std::string src = merge_sort_source(defs, less_expr, cuda_type_name<K>::get(), vt);
  unsigned long long nn = n;
  void *dummy_v = nullptr;
  void *vp = vals ? static_cast<void *>(vals) : dummy_v;
  {
    void *kp = keys;
    void *args[] = {&kp, &vp, &nn};
    jit_launch(src, "bcx_ms_block", unsigned((n + kMergeTile - 1) / kMergeTile), kMergeThreads, queue, args);
  }
  if (n <= kMergeTile) return;
  vector<K> tk(n, queue.get_context());
  vector<V> tv(vals ? n : 1, queue.get_context());
  K *ka = keys, *kb = tk.data();
  V *va = vals, *vb = vals ? tv.data() : nullptr;
  const unsigned grid = unsigned((n + size_t(kMergeTile) - 1) / kMergeTile);
  for (unsigned long long w = kMergeTile; w < n; w *= 2) {
    void *a0 = ka, *a1 = va, *a2 = kb, *a3 = vb;
    unsigned long long ww = w;
    void *args[] = {&a0, &a1, &a2, &a3, &nn, &ww};
    jit_launch(src, "bcx_ms_merge", grid, kMergeThreads, queue, args);
    std::swap(ka, kb);
    std::swap(va, vb);
  }
  if (ka != keys) {
    check(bcx_memcpy_async(keys, ka, n * sizeof(K), queue.get()));
    if (vals) check(bcx_memcpy_async(vals, va, n * sizeof(V), queue.get()));
  }
  queue.finish();  // the temporaries die here
}

}  // namespace detail
}  // namespace compute
}  // namespace boost

#endif
