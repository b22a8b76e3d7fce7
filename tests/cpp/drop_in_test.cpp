// Drop-in check: reference-style C++ callers compiled unchanged (apart from
// include paths) against the boost::compute headers of this repository and run
// on the GPU.  Each CHECK mirrors a known-answer test of the reference's test
// suite (file:line given); the program prints one line per failure and exits
// non-zero if any check failed.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <numeric>
#include <random>
#include <vector>

#include <boost/compute.hpp>
#include <boost/compute/container/mapped_view.hpp>
#include <boost/compute/iterator/zip_iterator.hpp>
#include <tuple>

namespace compute = boost::compute;

static int g_failures = 0;
#define CHECK(cond)                                                   \
  do {                                                                \
    if (!(cond)) {                                                    \
      std::printf("FAIL %s:%d: %s\n", __FILE__, __LINE__, #cond);     \
      ++g_failures;                                                   \
    }                                                                 \
  } while (0)

template <class T>
static std::vector<T> to_host(const compute::vector<T> &v, compute::command_queue &q) {
  std::vector<T> h(v.size());
  compute::copy(v.begin(), v.end(), h.begin(), q);
  return h;
}

// The README example: sort 2^20 random floats on the device.
static void readme_example() {
  compute::device gpu = compute::system::default_device();
  compute::context ctx(gpu);
  compute::command_queue queue(ctx, gpu);
  std::vector<float> host_vector(1 << 20);
  std::mt19937 gen(20261203);
  for (auto &x : host_vector) x = float(gen() % 2147483647u);
  compute::vector<float> device_vector(host_vector.size(), ctx);
  compute::copy(host_vector.begin(), host_vector.end(), device_vector.begin(), queue);
  compute::sort(device_vector.begin(), device_vector.end(), queue);
  std::vector<float> sorted(host_vector.size());
  compute::copy(device_vector.begin(), device_vector.end(), sorted.begin(), queue);
  std::vector<float> expect = host_vector;
  std::sort(expect.begin(), expect.end());
  CHECK(sorted == expect);
}

static void sort_cases(compute::command_queue &q) {
  // test/test_sort.cpp:135-145
  int data[] = {-4, 152, -5000, 963, 75321, -456, 0, 1112};
  compute::vector<int> v(data, data + 8, q);
  CHECK(!compute::is_sorted(v.begin(), v.end(), q));
  compute::sort(v.begin(), v.end(), q);
  CHECK((to_host(v, q) == std::vector<int>{-5000, -456, -4, 0, 152, 963, 1112, 75321}));
  // test/test_sort.cpp:227-236 (greater)
  compute::vector<int> r(data, data + 8, q);
  compute::sort(r.begin(), r.end(), compute::greater<int>(), q);
  CHECK((to_host(r, q) == std::vector<int>{75321, 1112, 963, 152, 0, -4, -456, -5000}));
  // test/test_sort.cpp:286-292 (host vector)
  std::vector<int> hv = {5, 2, 3, 6, 7, 4, 0, 1};
  compute::sort(hv.begin(), hv.end(), q);
  CHECK((hv == std::vector<int>{0, 1, 2, 3, 4, 5, 6, 7}));
  // test/test_radix_sort.cpp:530-543 (sub-range)
  int d2[] = {9, 8, 7, 6, 5, 4, 3, 2, 1, 0};
  compute::vector<int> p(d2, d2 + 10, q);
  compute::detail::radix_sort(p.begin() + 2, p.end() - 2, q);
  CHECK((to_host(p, q) == std::vector<int>{9, 8, 2, 3, 4, 5, 6, 7, 1, 0}));
  // test/test_radix_sort_by_key.cpp:30-61 (stability)
  int keys[] = {10, 9, 2, 7, 6, -1, 4, 2, 2, 10};
  int vals[] = {1, 2, 3, 4, 5, 6, 7, 8, 9, 10};
  compute::vector<int> k(keys, keys + 10, q), w(vals, vals + 10, q);
  compute::sort_by_key(k.begin(), k.end(), w.begin(), q);
  CHECK((to_host(k, q) == std::vector<int>{-1, 2, 2, 2, 4, 6, 7, 9, 10, 10}));
  CHECK((to_host(w, q) == std::vector<int>{6, 3, 8, 9, 7, 5, 4, 2, 1, 10}));
  // large stable sort_by_key
  const size_t n = 1000003;
  std::vector<compute::uint_> hk(n), hvals(n);
  std::mt19937 gen(1);
  for (size_t i = 0; i < n; ++i) { hk[i] = gen() % 1000; hvals[i] = compute::uint_(i); }
  compute::vector<compute::uint_> dk(hk.begin(), hk.end(), q), dv(hvals.begin(), hvals.end(), q);
  compute::stable_sort_by_key(dk.begin(), dk.end(), dv.begin(), q);
  std::vector<size_t> idx(n);
  std::iota(idx.begin(), idx.end(), size_t(0));
  std::stable_sort(idx.begin(), idx.end(), [&](size_t a, size_t b) { return hk[a] < hk[b]; });
  std::vector<compute::uint_> gk = to_host(dk, q), gv = to_host(dv, q);
  bool ok = true;
  for (size_t i = 0; i < n; ++i) ok = ok && gk[i] == hk[idx[i]] && gv[i] == compute::uint_(idx[i]);
  CHECK(ok);
}

static void scan_cases(compute::command_queue &q) {
  // test/test_scan.cpp:41-60 / 91-110
  int data[] = {0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11};
  compute::vector<int> v(data, data + 12, q), out(12, q.get_context());
  compute::inclusive_scan(v.begin(), v.end(), out.begin(), q);
  CHECK((to_host(out, q) == std::vector<int>{0, 1, 3, 6, 10, 15, 21, 28, 36, 45, 55, 66}));
  compute::exclusive_scan(v.begin(), v.end(), v.begin(), q);  // in place
  CHECK((to_host(v, q) == std::vector<int>{0, 0, 1, 3, 6, 10, 15, 21, 28, 36, 45, 55}));
  // test/test_scan.cpp:360-390 (multiplies, init 10)
  int m[] = {1, 2, 1, 2, 3};
  compute::vector<int> mv(m, m + 5, q), mo(5, q.get_context());
  compute::exclusive_scan(mv.begin(), mv.end(), mo.begin(), 10, compute::multiplies<int>(), q);
  CHECK((to_host(mo, q) == std::vector<int>{10, 10, 20, 20, 40}));
  // test/test_scan.cpp:190-222 (counting iterator input)
  compute::vector<int> c(10, q.get_context());
  compute::inclusive_scan(compute::make_counting_iterator(1), compute::make_counting_iterator(11), c.begin(), q);
  CHECK((to_host(c, q) == std::vector<int>{1, 3, 6, 10, 15, 21, 28, 36, 45, 55}));
}

static void reduce_cases(compute::command_queue &q) {
  // test/test_reduce.cpp:29-40
  int data[] = {1, 5, 9, 13, 17};
  compute::vector<int> v(data, data + 5, q);
  int sum = 0, product = 0;
  compute::reduce(v.begin(), v.end(), &sum, compute::plus<int>(), q);
  compute::reduce(v.begin(), v.end(), &product, compute::multiplies<int>(), q);
  CHECK(sum == 45);
  CHECK(product == 9945);
  // test/test_reduce.cpp:80-88 (device result)
  int d8[] = {1, 2, 3, 4, 5, 6, 7, 8};
  compute::vector<int> in(d8, d8 + 8, q), res(2, q.get_context());
  compute::reduce(in.begin(), in.begin() + 4, res.begin(), q);
  compute::reduce(in.begin() + 4, in.end(), res.end() - 1, q);
  CHECK((to_host(res, q) == std::vector<int>{10, 26}));
  // test/test_reduce.cpp:42-49 (empty leaves the result alone)
  compute::vector<short> empty(q.get_context());
  short s = 0;
  compute::reduce(empty.begin(), empty.end(), &s, q);
  CHECK(s == 0);
  // test/test_accumulate.cpp:25-85
  int a[] = {2, 4, 6, 8};
  compute::vector<int> av(a, a + 4, q);
  CHECK(compute::accumulate(av.begin(), av.end(), 0, q) == 20);
  CHECK(compute::accumulate(av.begin(), av.end(), -10, q) == 10);
  CHECK(compute::accumulate(av.begin(), av.end(), 2, compute::multiplies<int>(), q) == 768);
  int qd[] = {2, 8, 16};
  compute::vector<int> qv(qd, qd + 3, q);
  CHECK(compute::accumulate(qv.begin(), qv.end(), 1024, compute::divides<int>(), q) == 4);
  // test/test_accumulate.cpp:150-206 (iota sums)
  compute::vector<int> io(1025, q.get_context());
  compute::iota(io.begin(), io.end(), 0, q);
  CHECK(compute::accumulate(io.begin(), io.end(), 2, q) == 524802);
}

static void transform_cases(compute::command_queue &q) {
  // test/test_transform.cpp:29-41
  int data[] = {1, -2, -3, -4, 5};
  compute::vector<int> v(data, data + 5, q);
  compute::transform(v.begin(), v.end(), v.begin(), compute::abs<int>(), q);
  CHECK((to_host(v, q) == std::vector<int>{1, 2, 3, 4, 5}));
  // test/test_transform.cpp:75-99
  int d1[] = {1, 2, 3, 4}, d2[] = {10, 20, 30, 40};
  compute::vector<int> i1(d1, d1 + 4, q), i2(d2, d2 + 4, q), o(4, q.get_context());
  compute::transform(i1.begin(), i1.end(), i2.begin(), o.begin(), compute::plus<int>(), q);
  CHECK((to_host(o, q) == std::vector<int>{11, 22, 33, 44}));
}

static void reduce_by_key_cases(compute::command_queue &q) {
  // test/test_reduce_by_key.cpp:26-46
  int keys[] = {0, 2, -3, -3, -3, -3, -3, 4};
  int data[] = {1, 1, 1, 1, 1, 2, 5, 1};
  compute::vector<int> ki(keys, keys + 8, q), vi(data, data + 8, q), ko(8, q.get_context()), vo(8, q.get_context());
  auto ends = compute::reduce_by_key(ki.begin(), ki.end(), vi.begin(), ko.begin(), vo.begin(), q);
  CHECK(ends.first - ko.begin() == 4);
  std::vector<int> hk = to_host(ko, q), hv = to_host(vo, q);
  CHECK((std::vector<int>(hk.begin(), hk.begin() + 4) == std::vector<int>{0, 2, -3, 4}));
  CHECK((std::vector<int>(hv.begin(), hv.begin() + 4) == std::vector<int>{1, 1, 10, 1}));
  // run keys discarded
  compute::vector<int> vo2(8, q.get_context());
  auto ends2 = compute::reduce_by_key(ki.begin(), ki.end(), vi.begin(), compute::make_discard_iterator(),
                                      vo2.begin(), compute::plus<int>(), q);
  CHECK(ends2.first.get_index() == 4 && ends2.second - vo2.begin() == 4);
  std::vector<int> hv2 = to_host(vo2, q);
  CHECK((std::vector<int>(hv2.begin(), hv2.begin() + 4) == std::vector<int>{1, 1, 10, 1}));
}

static void jit_cases(compute::command_queue &q) {
  using compute::_1;
  using compute::_2;
  // perf/perf_saxpy.cpp:50-56: alpha * _1 + _2 (one rounding, like fmaf)
  const size_t n = (1 << 20) + 3;
  std::vector<float> hx(n), hy(n);
  std::mt19937 gen(5);
  std::uniform_real_distribution<float> u(-1.f, 1.f);
  for (size_t i = 0; i < n; ++i) { hx[i] = u(gen); hy[i] = u(gen); }
  compute::vector<float> x(hx.begin(), hx.end(), q), y(hy.begin(), hy.end(), q), r(n, q.get_context());
  const float alpha = 2.5f;
  compute::transform(x.begin(), x.end(), y.begin(), r.begin(), alpha * _1 + _2, q);
  std::vector<float> hr = to_host(r, q);
  bool exact = true;
  for (size_t i = 0; i < n; ++i) exact = exact && hr[i] == std::fma(alpha, hx[i], hy[i]);
  CHECK(exact);
  // test/test_transform.cpp:61-73 (clamp)
  float cd[] = {10.f, 20.f, 30.f, 40.f, 50.f};
  compute::vector<float> cv(cd, cd + 5, q);
  compute::transform(cv.begin(), cv.end(), cv.begin(), clamp(_1, 15.f, 45.f), q);
  CHECK((to_host(cv, q) == std::vector<float>{15.f, 20.f, 30.f, 40.f, 45.f}));
  // test/test_transform.cpp:101-118 (pown)
  float pd[] = {1.f, 2.f, 3.f, 4.f};
  compute::vector<float> pv(pd, pd + 4, q), po(4, q.get_context());
  compute::transform(pv.begin(), pv.end(), po.begin(), pown(_1, 4), q);
  CHECK((to_host(po, q) == std::vector<float>{1.f, 16.f, 81.f, 256.f}));
  // test/test_transform.cpp:120-141 (BOOST_COMPUTE_FUNCTION)
  float fd[] = {9.f, 7.f, 5.f, 3.f};
  compute::vector<float> fv(fd, fd + 4, q), fo(4, q.get_context());
  BOOST_COMPUTE_FUNCTION(float, pow3add4, (float x), { return pow(x, 3.0f) + 4.0f; });
  compute::transform(fv.begin(), fv.end(), fo.begin(), pow3add4, q);
  std::vector<float> hfo = to_host(fo, q);
  CHECK(std::fabs(hfo[0] - 733.f) < 1e-3f && std::fabs(hfo[3] - 31.f) < 1e-4f);
  // test/test_closure.cpp:32-47 (BOOST_COMPUTE_CLOSURE)
  int two = 2;
  BOOST_COMPUTE_CLOSURE(int, add_two, (int x), (two), { return x + two; });
  int id[] = {1, 2, 3, 4};
  compute::vector<int> iv(id, id + 4, q);
  compute::transform(iv.begin(), iv.end(), iv.begin(), add_two, q);
  CHECK((to_host(iv, q) == std::vector<int>{3, 4, 5, 6}));
  // test/test_scan.cpp:438-488 (custom function scans)
  BOOST_COMPUTE_FUNCTION(int, multi, (int x, int y), { return x * y * 2; });
  int sd[] = {1, 2, 1, 2, 3};
  compute::vector<int> sv(sd, sd + 5, q), so(5, q.get_context());
  compute::inclusive_scan(sv.begin(), sv.end(), so.begin(), multi, q);
  CHECK((to_host(so, q) == std::vector<int>{1, 4, 8, 32, 192}));
  compute::exclusive_scan(sv.begin(), sv.end(), so.begin(), 1, multi, q);
  CHECK((to_host(so, q) == std::vector<int>{1, 2, 8, 16, 64}));
  compute::exclusive_scan(sv.begin(), sv.end(), sv.begin(), 1, multi, q);  // in place
  CHECK((to_host(sv, q) == std::vector<int>{1, 2, 8, 16, 64}));
  // test/test_scan.cpp:258-285 (scan of a transform_iterator)
  float td[] = {1.f, 2.f, 3.f, 4.f, 5.f};
  compute::vector<float> tv(td, td + 5, q), to(5, q.get_context());
  compute::inclusive_scan(compute::make_transform_iterator(tv.begin(), pown(_1, 2)),
                          compute::make_transform_iterator(tv.end(), pown(_1, 2)), to.begin(), q);
  CHECK((to_host(to, q) == std::vector<float>{1.f, 5.f, 14.f, 30.f, 55.f}));
  // a user functor in reduce/accumulate (associative)
  BOOST_COMPUTE_FUNCTION(int, add3, (int a, int b), { return a + b; });
  compute::vector<int> big(100003, q.get_context());
  compute::iota(big.begin(), big.end(), 0, q);
  CHECK(compute::accumulate(big.begin(), big.end(), 5, add3, q) == int(5 + (100003LL * 100002 / 2) % (1LL << 32)));
  // a build failure surfaces as program_build_failure with the log
  BOOST_COMPUTE_FUNCTION(int, broken, (int x), { return x +; });
  bool threw = false;
  try {
    compute::transform(iv.begin(), iv.end(), iv.begin(), broken, q);
  } catch (const compute::program_build_failure &e) {
    threw = !e.build_log().empty();
  }
  CHECK(threw);
}

// User functors on the generated single-pass scan and one-launch fold, at
// sizes with many tiles (look-back across tiles, in-order folds across blocks).
static void jit_large_cases(compute::command_queue &q) {
  // test/test_scan.cpp:414-436 (exclusive multiplies, init 10, 1000 twos) with
  // the functor given as a user function instead of multiplies<int>
  BOOST_COMPUTE_FUNCTION(int, times, (int x, int y), { return x * y; });
  compute::vector<int> tw(1000, 2, q);
  compute::exclusive_scan(tw.begin(), tw.end(), tw.begin(), 10, times, q);
  std::vector<int> expect_tw(1000, 2);
  expect_tw[0] = 10;
  {
    unsigned run = 1;
    for (size_t i = 0; i < expect_tw.size(); ++i) {
      run *= unsigned(expect_tw[i]);
      expect_tw[i] = int(run);
    }
  }
  CHECK(to_host(tw, q) == expect_tw);
  // inclusive plus through a user function over 3,000,017 elements (wraps)
  const size_t n = 3000017;
  std::vector<int> h(n);
  for (size_t i = 0; i < n; ++i) h[i] = int(i % 1000) - 500 + int((i * 2654435761u) >> 28);
  BOOST_COMPUTE_FUNCTION(int, add_u, (int a, int b), { return (int)((unsigned)a + (unsigned)b); });
  compute::vector<int> dv(h.begin(), h.end(), q), dout(n, q.get_context());
  compute::inclusive_scan(dv.begin(), dv.end(), dout.begin(), add_u, q);
  std::vector<int> ref(n);
  {
    unsigned run = 0;
    for (size_t i = 0; i < n; ++i) {
      run += unsigned(h[i]);
      ref[i] = int(run);
    }
  }
  CHECK(to_host(dout, q) == ref);
  // exclusive, init 7, in place
  compute::exclusive_scan(dv.begin(), dv.end(), dv.begin(), 7, add_u, q);
  {
    unsigned run = 7;
    for (size_t i = 0; i < n; ++i) {
      const unsigned x = unsigned(h[i]);
      ref[i] = int(run);
      run += x;
    }
  }
  CHECK(to_host(dv, q) == ref);
  // a non-commutative associative functor on a 16-byte type: products of
  // 2x2 integer matrices mod 2^32, scanned and folded in input order
  BOOST_COMPUTE_FUNCTION(compute::int4_, matmul, (compute::int4_ a, compute::int4_ b), {
    const unsigned a0 = a.x, a1 = a.y, a2 = a.z, a3 = a.w, b0 = b.x, b1 = b.y, b2 = b.z, b3 = b.w;
    return make_int4((int)(a0 * b0 + a1 * b2), (int)(a0 * b1 + a1 * b3), (int)(a2 * b0 + a3 * b2),
                     (int)(a2 * b1 + a3 * b3));
  });
  const size_t m = 1000003;
  std::vector<compute::int4_> hm(m);
  std::mt19937 gen(7);
  for (size_t i = 0; i < m; ++i)
    hm[i] = compute::int4_(int(gen() % 4) - 1, int(gen() % 4) - 1, int(gen() % 4) - 1, int(gen() % 4) - 1);
  auto mul = [](const compute::int4_ &a, const compute::int4_ &b) {
    const unsigned a0 = a[0], a1 = a[1], a2 = a[2], a3 = a[3], b0 = b[0], b1 = b[1], b2 = b[2], b3 = b[3];
    return compute::int4_(int(a0 * b0 + a1 * b2), int(a0 * b1 + a1 * b3), int(a2 * b0 + a3 * b2),
                          int(a2 * b1 + a3 * b3));
  };
  compute::vector<compute::int4_> dm(hm.begin(), hm.end(), q), dmo(m, q.get_context());
  compute::inclusive_scan(dm.begin(), dm.end(), dmo.begin(), matmul, q);
  std::vector<compute::int4_> got = to_host(dmo, q);
  std::vector<compute::int4_> pref(m);
  pref[0] = hm[0];
  for (size_t i = 1; i < m; ++i) pref[i] = mul(pref[i - 1], hm[i]);
  CHECK(got == pref);
  compute::vector<compute::int4_> fold(1, q.get_context());
  compute::reduce(dm.begin(), dm.end(), fold.begin(), matmul, q);
  CHECK(fold.begin().read(q) == pref[m - 1]);
}

// The staged generated scan (whole tiles bulk-copied through shared memory)
// at its edges: 1- and 2-byte elements whose last tile ends in a ragged tail
// under 16 bytes, 8-byte elements (96 KB tiles), a non-commutative functor,
// in place, and an input one element off 16-byte alignment (which takes the
// register-tile kernel instead).
static void jit_staged_cases(compute::command_queue &q) {
  std::mt19937 gen(11);
  {
    const size_t n = 300001;  // 4.6 tiles of 64 KB, 1-byte tail
    std::vector<unsigned char> h(n);
    for (auto &x : h) x = (unsigned char)(gen() & 0xff);
    BOOST_COMPUTE_FUNCTION(compute::uchar_, bxor, (compute::uchar_ a, compute::uchar_ b), { return (uchar_)(a ^ b); });
    compute::vector<unsigned char> d(h.begin(), h.end(), q), o(n, q.get_context());
    compute::inclusive_scan(d.begin(), d.end(), o.begin(), bxor, q);
    std::vector<unsigned char> ref(n);
    unsigned char run = 0;
    for (size_t i = 0; i < n; ++i) ref[i] = run = (unsigned char)(run ^ h[i]);
    CHECK(to_host(o, q) == ref);
  }
  {
    const size_t n = 777777;  // "last nonzero" is associative, not commutative
    std::vector<short> h(n);
    for (auto &x : h) x = (gen() % 5 == 0) ? short(gen() % 2001) - 1000 : short(0);
    BOOST_COMPUTE_FUNCTION(compute::short_, last_nz, (compute::short_ a, compute::short_ b), { return b != 0 ? b : a; });
    compute::vector<short> d(h.begin(), h.end(), q);
    compute::exclusive_scan(d.begin(), d.end(), d.begin(), short(-7), last_nz, q);  // in place
    std::vector<short> ref(n);
    short run = -7;
    for (size_t i = 0; i < n; ++i) {
      ref[i] = run;
      if (h[i] != 0) run = h[i];
    }
    CHECK(to_host(d, q) == ref);
  }
  {
    const size_t n = 1000003;  // 81.4 tiles of 96 KB, one element in the tail
    std::vector<int64_t> h(n);
    for (auto &x : h) x = int64_t(gen() % 2000001) - 1000000;
    BOOST_COMPUTE_FUNCTION(compute::long_, add_l, (compute::long_ a, compute::long_ b), { return a + b; });
    compute::vector<int64_t> d(h.begin(), h.end(), q), o(n, q.get_context());
    compute::exclusive_scan(d.begin(), d.end(), o.begin(), int64_t(-3), add_l, q);
    std::vector<int64_t> ref(n);
    int64_t run = -3;
    for (size_t i = 0; i < n; ++i) {
      ref[i] = run;
      run += h[i];
    }
    CHECK(to_host(o, q) == ref);
    // one element off 16-byte alignment: the register-tile kernel
    compute::inclusive_scan(d.begin() + 1, d.end(), o.begin() + 1, add_l, q);
    std::vector<int64_t> got = to_host(o, q);
    run = 0;
    bool ok = true;
    for (size_t i = 1; i < n; ++i) {
      run += h[i];
      ok = ok && got[i] == run;
    }
    CHECK(ok);
  }
}

// zip_iterator, mapped_view and accumulate with an init of another type.
static void zip_view_cases(compute::command_queue &q) {
  // test/test_zip_iterator.cpp:47-105 (distance)
  compute::vector<char> cvec(5, q.get_context());
  compute::vector<int> ivec(5, q.get_context());
  CHECK(std::distance(compute::make_zip_iterator(std::make_tuple(cvec.begin(), ivec.begin())),
                      compute::make_zip_iterator(std::make_tuple(cvec.end(), ivec.end()))) == 5);
  // test/test_zip_iterator.cpp:107-155 (copy three vectors into a vector of tuples)
  char cd[] = {'x', 'y', 'z'};
  int id[] = {4, 7, 9};
  float fd[] = {3.2f, 4.5f, 7.6f};
  compute::vector<char> cv(cd, cd + 3, q);
  compute::vector<int> iv(id, id + 3, q);
  compute::vector<float> fv(fd, fd + 3, q);
  compute::vector<std::tuple<char, int, float> > tv(3, q.get_context());
  compute::copy(compute::make_zip_iterator(std::make_tuple(cv.begin(), iv.begin(), fv.begin())),
                compute::make_zip_iterator(std::make_tuple(cv.end(), iv.end(), fv.end())), tv.begin(), q);
  std::vector<std::tuple<char, int, float> > ht = to_host(tv, q);
  CHECK(ht.size() == 3 && ht[0] == std::make_tuple('x', 4, 3.2f) && ht[1] == std::make_tuple('y', 7, 4.5f) &&
        ht[2] == std::make_tuple('z', 9, 7.6f));
  // test/test_zip_iterator.cpp:157-207 (transform with get<N>)
  int d1[] = {0, 2, 4, 6, 8};
  int d2[] = {1, 3, 5, 7, 9};
  compute::vector<int> in1(d1, d1 + 5, q), in2(d2, d2 + 5, q), out(5, q.get_context());
  compute::transform(compute::make_zip_iterator(std::make_tuple(in1.begin())),
                     compute::make_zip_iterator(std::make_tuple(in1.end())), out.begin(), compute::get<0>(), q);
  CHECK((to_host(out, q) == std::vector<int>{0, 2, 4, 6, 8}));
  compute::transform(compute::make_zip_iterator(std::make_tuple(in2.begin(), in1.begin())),
                     compute::make_zip_iterator(std::make_tuple(in2.end(), in1.end())), out.begin(),
                     compute::get<1>(), q);
  CHECK((to_host(out, q) == std::vector<int>{0, 2, 4, 6, 8}));
  // three ranges into a user function of the tuple
  BOOST_COMPUTE_FUNCTION(float, fma3, (std::tuple<float, float, float> t),
                         { return boost_tuple_get(t, 0) * boost_tuple_get(t, 1) + boost_tuple_get(t, 2); });
  float a3[] = {1.f, 2.f, 3.f}, b3[] = {4.f, 5.f, 6.f}, c3[] = {0.5f, 0.25f, 0.125f};
  compute::vector<float> va(a3, a3 + 3, q), vb(b3, b3 + 3, q), vc(c3, c3 + 3, q), vr(3, q.get_context());
  compute::transform(compute::make_zip_iterator(std::make_tuple(va.begin(), vb.begin(), vc.begin())),
                     compute::make_zip_iterator(std::make_tuple(va.end(), vb.end(), vc.end())), vr.begin(), fma3, q);
  CHECK((to_host(vr, q) == std::vector<float>{4.5f, 10.25f, 18.125f}));
  // the lambda form, get<0>(_1) < 5, in count_if (test/test_count.cpp:182)
  using compute::lambda::get;
  CHECK(compute::count_if(compute::make_zip_iterator(std::make_tuple(in1.begin(), in2.begin())),
                          compute::make_zip_iterator(std::make_tuple(in1.end(), in2.end())),
                          get<0>(compute::_1) < 5, q) == 3);
  // test/test_accumulate.cpp:258-299 (std::accumulate equality through a
  // mapped_view, int init over int, float and double data)
  std::vector<int> h1 = {1, 2, 3, 4};
  {
    compute::mapped_view<int> view(h1.data(), h1.size(), q.get_context());
    CHECK(compute::accumulate(view.begin(), view.end(), 0, q) == std::accumulate(h1.begin(), h1.end(), 0));
  }
  h1.assign(10000, 2);
  {
    compute::mapped_view<int> view(h1.data(), h1.size(), q.get_context());
    CHECK(compute::accumulate(view.begin(), view.end(), 0, q) == std::accumulate(h1.begin(), h1.end(), 0));
  }
  std::vector<float> h2 = {1.2f, 2.3f, 4.5f, 6.7f, 8.9f};
  {
    compute::mapped_view<float> view(h2.data(), h2.size(), q.get_context());
    CHECK(compute::accumulate(view.begin(), view.end(), 0, q) == std::accumulate(h2.begin(), h2.end(), 0));
  }
  h2.assign(10000, 1.01f);
  {
    compute::mapped_view<float> view(h2.data(), h2.size(), q.get_context());
    CHECK(compute::accumulate(view.begin(), view.end(), 0, q) == std::accumulate(h2.begin(), h2.end(), 0));
  }
  std::vector<double> h3(10000, 2.02);
  {
    compute::mapped_view<double> view(h3.data(), h3.size(), q.get_context());
    CHECK(compute::accumulate(view.begin(), view.end(), 0, q) == std::accumulate(h3.begin(), h3.end(), 0));
  }
  // a device sort writing through a mapped view into host memory
  std::vector<int> hs(100003);
  std::mt19937 gen(3);
  for (auto &x : hs) x = int(gen() % 1000000) - 500000;
  std::vector<int> expect = hs;
  std::sort(expect.begin(), expect.end());
  {
    compute::mapped_view<int> view(hs.data(), hs.size(), q.get_context());
    compute::sort(view.begin(), view.end(), q);
    view.map(q);
  }
  CHECK(hs == expect);
}

static void transform_reduce_cases(compute::command_queue &q) {
  using compute::_1;
  using compute::_2;
  // test/test_transform_reduce.cpp:27-45 (sum of absolute values)
  int ad[] = {1, -2, 3, -4, 5};
  compute::vector<int> av(ad, ad + 5, q);
  int sum = 0;
  compute::transform_reduce(av.begin(), av.end(), &sum, compute::abs<int>(), compute::plus<int>(), q);
  CHECK(sum == 15);
  // lambda transform, device result
  float fd[] = {1.f, 2.f, 3.f, 4.f};
  compute::vector<float> fv(fd, fd + 4, q), fr(1, q.get_context());
  compute::transform_reduce(fv.begin(), fv.end(), fr.begin(), _1 * _1, compute::plus<float>(), q);
  CHECK(fr.begin().read(q) == 30.f);
  // binary form: dot product of 2^20 + 7 integers (exact, wraps mod 2^32)
  const size_t n = (1 << 20) + 7;
  std::vector<int> ha(n), hb(n);
  unsigned long long expect = 0;
  for (size_t i = 0; i < n; ++i) {
    ha[i] = int(i % 1000) - 500;
    hb[i] = int((i * 7) % 300);
    expect += (unsigned long long)(long long)(ha[i] * hb[i]);
  }
  compute::vector<int> a(ha.begin(), ha.end(), q), b(hb.begin(), hb.end(), q);
  int dot = 0;
  compute::transform_reduce(a.begin(), a.end(), b.begin(), &dot, compute::multiplies<int>(), compute::plus<int>(), q);
  CHECK(dot == int(unsigned(expect)));
  // user function transform, built-in max reduce
  BOOST_COMPUTE_FUNCTION(int, sq_minus, (int x), { return x * x - 10; });
  int mx = 0;
  compute::transform_reduce(av.begin(), av.end(), &mx, sq_minus, compute::max<int>(), q);
  CHECK(mx == 15);
  // binary lambda transform, lambda reduce
  compute::vector<int> r1(1, q.get_context());
  compute::transform_reduce(a.begin(), a.begin() + 4, b.begin(), r1.begin(), _1 - _2, _1 + _2, q);
  CHECK(r1.begin().read(q) == (-500 - 0) + (-499 - 7) + (-498 - 14) + (-497 - 21));
}

static void scan_family_cases(compute::command_queue &q) {
  using compute::_1;
  using compute::_2;
  // test/test_count.cpp (count / count_if with a lambda)
  int cd[] = {1, 2, 1, 2, 3, 1, 4, 1};
  compute::vector<int> cv(cd, cd + 8, q);
  CHECK(compute::count(cv.begin(), cv.end(), 1, q) == 4);
  CHECK(compute::count(cv.begin(), cv.end(), 5, q) == 0);
  CHECK(compute::count_if(cv.begin(), cv.end(), _1 > 1, q) == 4);
  BOOST_COMPUTE_FUNCTION(bool, is_odd, (int x), { return x & 1; });
  CHECK(compute::count_if(cv.begin(), cv.end(), is_odd, q) == 5);
  // a large count: 2^20 + 5 elements, every third one matches
  const size_t n = (1 << 20) + 5;
  std::vector<int> big(n);
  for (size_t i = 0; i < n; ++i) big[i] = int(i % 3);
  compute::vector<int> bv(big.begin(), big.end(), q);
  CHECK(compute::count(bv.begin(), bv.end(), 0, q) == (n + 2) / 3);
  // inner_product (test/test_inner_product.cpp)
  int ad[] = {1, 2, 3, 4}, bd[] = {5, 6, 7, 8};
  compute::vector<int> a(ad, ad + 4, q), b(bd, bd + 4, q);
  CHECK(compute::inner_product(a.begin(), a.end(), b.begin(), 10, q) == 10 + 70);
  CHECK(compute::inner_product(a.begin(), a.end(), b.begin(), 0, compute::plus<int>(), compute::minus<int>(), q) == -16);
  // min_element / max_element return the FIRST extremum (test/test_extrema.cpp)
  int ed[] = {9, 15, 1, 4, 1, 15, 9, 0, 0, 12};
  compute::vector<int> ev(ed, ed + 10, q);
  CHECK(compute::min_element(ev.begin(), ev.end(), q) - ev.begin() == 7);
  CHECK(compute::max_element(ev.begin(), ev.end(), q) - ev.begin() == 1);
  CHECK(compute::min_element(ev.begin(), ev.end(), compute::greater<int>(), q) - ev.begin() == 1);
  CHECK(compute::max_element(ev.begin(), ev.end(), _1 > _2, q) - ev.begin() == 7);
  std::vector<float> fx(n);
  for (size_t i = 0; i < n; ++i) fx[i] = float((i * 7919) % 100003);
  fx[123457] = -5.f;
  fx[999999] = -5.f;
  fx[54321] = 200000.f;
  compute::vector<float> fv(fx.begin(), fx.end(), q);
  CHECK(compute::min_element(fv.begin(), fv.end(), q) - fv.begin() == 123457);
  CHECK(compute::max_element(fv.begin(), fv.end(), q) - fv.begin() == 54321);
  // copy_if / remove_copy_if keep order (test/test_copy_if.cpp)
  int xd[] = {1, 6, 2, 7, 3, 8, 4, 9, 5};
  compute::vector<int> xv(xd, xd + 9, q), out(9, q.get_context());
  auto end = compute::copy_if(xv.begin(), xv.end(), out.begin(), _1 > 4, q);
  CHECK(end - out.begin() == 5);
  std::vector<int> ho = to_host(out, q);
  CHECK((std::vector<int>(ho.begin(), ho.begin() + 5) == std::vector<int>{6, 7, 8, 9, 5}));
  end = compute::remove_copy_if(xv.begin(), xv.end(), out.begin(), _1 > 4, q);
  ho = to_host(out, q);
  CHECK(end - out.begin() == 4 && (std::vector<int>(ho.begin(), ho.begin() + 4) == std::vector<int>{1, 2, 3, 4}));
  compute::vector<int> bo(n, q.get_context());
  auto bend = compute::copy_if(bv.begin(), bv.end(), bo.begin(), _1 == 2, q);
  CHECK(size_t(bend - bo.begin()) == n / 3);
  std::vector<int> hb = to_host(bo, q);
  bool all2 = true;
  for (size_t i = 0; i < n / 3; ++i) all2 = all2 && hb[i] == 2;
  CHECK(all2);
}

static void compaction_cases(compute::command_queue &q) {
  using compute::_1;
  using compute::_2;
  // test/test_unique.cpp
  int ud[] = {1, 1, 2, 2, 2, 3, 1, 1, 5};
  compute::vector<int> uv(ud, ud + 9, q);
  auto uend = compute::unique(uv.begin(), uv.end(), q);
  std::vector<int> hu = to_host(uv, q);
  CHECK(uend - uv.begin() == 5 && (std::vector<int>(hu.begin(), hu.begin() + 5) == std::vector<int>{1, 2, 3, 1, 5}));
  // unique_copy with a custom predicate: runs of elements within 1 of their predecessor
  int cd[] = {10, 11, 12, 20, 21, 30, 31, 32, 33};
  compute::vector<int> cv(cd, cd + 9, q), co(9, q.get_context());
  BOOST_COMPUTE_FUNCTION(bool, close_to, (int a, int b), { return b - a == 1; });
  auto cend = compute::unique_copy(cv.begin(), cv.end(), co.begin(), close_to, q);
  std::vector<int> hc = to_host(co, q);
  CHECK(cend - co.begin() == 3 && (std::vector<int>(hc.begin(), hc.begin() + 3) == std::vector<int>{10, 20, 30}));
  // stable_partition keeps both halves in input order (test/test_stable_partition.cpp)
  int pd[] = {1, 2, 3, 4, 5, 6, 7, 8, 9, 10};
  compute::vector<int> pv(pd, pd + 10, q);
  auto mid = compute::stable_partition(pv.begin(), pv.end(), _1 % 2 == 0, q);
  CHECK(mid - pv.begin() == 5);
  CHECK((to_host(pv, q) == std::vector<int>{2, 4, 6, 8, 10, 1, 3, 5, 7, 9}));
  // remove_if / remove (test/test_remove.cpp)
  int rd[] = {1, 5, 2, 5, 3, 5, 4};
  compute::vector<int> rv(rd, rd + 7, q);
  auto rend = compute::remove(rv.begin(), rv.end(), 5, q);
  std::vector<int> hr = to_host(rv, q);
  CHECK(rend - rv.begin() == 4 && (std::vector<int>(hr.begin(), hr.begin() + 4) == std::vector<int>{1, 2, 3, 4}));
  compute::vector<int> rv2(rd, rd + 7, q);
  auto rend2 = compute::remove_if(rv2.begin(), rv2.end(), _1 < 3, q);
  std::vector<int> hr2 = to_host(rv2, q);
  CHECK(rend2 - rv2.begin() == 5 && (std::vector<int>(hr2.begin(), hr2.begin() + 5) == std::vector<int>{5, 5, 3, 5, 4}));
  // a large unique: 2^20 + 9 elements in runs of 3
  const size_t n = (1 << 20) + 9;
  std::vector<int> big(n);
  for (size_t i = 0; i < n; ++i) big[i] = int(i / 3);
  compute::vector<int> bv(big.begin(), big.end(), q);
  auto bend = compute::unique(bv.begin(), bv.end(), q);
  CHECK(size_t(bend - bv.begin()) == (n + 2) / 3);
  std::vector<int> hb = to_host(bv, q);
  bool ok = true;
  for (size_t i = 0; i < (n + 2) / 3; ++i) ok = ok && hb[i] == int(i);
  CHECK(ok);
}

static void comparator_sort_cases(compute::command_queue &q) {
  using compute::_1;
  using compute::_2;
  // test/test_sort.cpp: sort with a lambda comparator (descending)
  int d[] = {3, 9, -1, 4, 4, 0, 7};
  compute::vector<int> v(d, d + 7, q);
  compute::sort(v.begin(), v.end(), _1 > _2, q);
  CHECK((to_host(v, q) == std::vector<int>{9, 7, 4, 4, 3, 0, -1}));
  // stable_sort_by_key with a user comparator on |key|: ties keep input order
  BOOST_COMPUTE_FUNCTION(bool, abs_less, (int a, int b), { return abs(a) < abs(b); });
  const size_t n = (1 << 20) + 3;
  std::mt19937 gen(7);
  std::uniform_int_distribution<int> dist(-5000, 5000);
  std::vector<int> hk(n), hv(n);
  for (size_t i = 0; i < n; ++i) {
    hk[i] = dist(gen);
    hv[i] = int(i);
  }
  compute::vector<int> k(hk.begin(), hk.end(), q), val(hv.begin(), hv.end(), q);
  compute::stable_sort_by_key(k.begin(), k.end(), val.begin(), abs_less, q);
  std::vector<size_t> idx(n);
  for (size_t i = 0; i < n; ++i) idx[i] = i;
  std::stable_sort(idx.begin(), idx.end(), [&](size_t a, size_t b) { return std::abs(hk[a]) < std::abs(hk[b]); });
  std::vector<int> gk = to_host(k, q), gv = to_host(val, q);
  bool same = true;
  for (size_t i = 0; i < n; ++i) same = same && gk[i] == hk[idx[i]] && gv[i] == int(idx[i]);
  CHECK(same);
  // keys only, float, lambda comparator, 3 * 2^18 + 5 elements
  const size_t m = 3 * (1 << 18) + 5;
  std::vector<float> hf(m);
  std::uniform_real_distribution<float> u(-1.f, 1.f);
  for (size_t i = 0; i < m; ++i) hf[i] = u(gen);
  compute::vector<float> fv(hf.begin(), hf.end(), q);
  compute::sort(fv.begin(), fv.end(), _1 < _2, q);
  std::sort(hf.begin(), hf.end());
  CHECK(to_host(fv, q) == hf);
}

static void error_cases(compute::command_queue &q) {
  // bcx errors surface as opencl_error with the OpenCL status code
  bool thrown = false;
  try {
    compute::detail::check(bcx_scan(q.get(), bcx_dtype(42), BCX_PLUS, 0, nullptr, nullptr, nullptr, 1, 0, nullptr,
                                    nullptr));
  } catch (const compute::opencl_error &e) {
    thrown = e.error_code() == -30;
  }
  CHECK(thrown);
}

// copy_async / fill_async / futures / events.
static void async_cases(compute::command_queue &q) {
  // test_copy.cpp:219 copy_int_async
  int host_data[] = {1, 2, 3, 4, 5, 6, 7, 8};
  compute::vector<int> device_data(8, q.get_context());
  compute::future<compute::vector<int>::iterator> h2d =
      compute::copy_async(host_data, host_data + 8, device_data.begin(), q);
  h2d.wait();
  CHECK((to_host(device_data, q) == std::vector<int>{1, 2, 3, 4, 5, 6, 7, 8}));
  CHECK(h2d.get() == device_data.end());
  std::fill(host_data, host_data + 8, 0);
  compute::future<int *> d2h = compute::copy_async(device_data.begin(), device_data.end(), host_data, q);
  d2h.wait();
  CHECK((std::vector<int>(host_data, host_data + 8) == std::vector<int>{1, 2, 3, 4, 5, 6, 7, 8}));
  CHECK(d2h.get() == host_data + 8);

  // test_async_wait.cpp:29 wait_for_copy: fill_async, then four pieces copied
  // independently and waited for together
  compute::vector<int> v(8, q.get_context());
  compute::future<void> fill_future = compute::fill_async(v.begin(), v.end(), 9, q);
  compute::wait_for_all(fill_future);
  CHECK((to_host(v, q) == std::vector<int>(8, 9)));
  int data[] = {1, 2, 3, 4, 5, 6, 7, 8};
  auto c1 = compute::copy_async(data + 0, data + 2, v.begin() + 0, q);
  auto c2 = compute::copy_async(data + 2, data + 4, v.begin() + 2, q);
  auto c3 = compute::copy_async(data + 4, data + 6, v.begin() + 4, q);
  auto c4 = compute::copy_async(data + 6, data + 8, v.begin() + 6, q);
  compute::wait_for_all(c1, c2, c3, c4);
  CHECK((to_host(v, q) == std::vector<int>{1, 2, 3, 4, 5, 6, 7, 8}));

  // fill with a value whose bytes differ (doubling copies) and a ragged size
  compute::vector<float> f(1000, q.get_context());
  compute::fill(f.begin(), f.end(), 1.5f, q);
  CHECK((to_host(f, q) == std::vector<float>(1000, 1.5f)));
  compute::vector<int> pat(12345, q.get_context());
  compute::fill_async(pat.begin(), pat.end(), 0x01020304, q).wait();
  CHECK((to_host(pat, q) == std::vector<int>(12345, 0x01020304)));
  compute::fill(pat.begin(), pat.end(), -1, q);  // one byte pattern: memset
  CHECK((to_host(pat, q) == std::vector<int>(12345, -1)));

  // page-locked host memory: the copy overlaps, its event times it, and a
  // second queue waits for it on the device before reducing the data
  const size_t n = size_t(1) << 24;
  void *pinned = nullptr;
  CHECK(bcx_malloc_host(&pinned, n * sizeof(int)) == BCX_SUCCESS);
  if (pinned) {
    int *hp = static_cast<int *>(pinned);
    for (size_t i = 0; i < n; ++i) hp[i] = int(i % 7);
    compute::vector<int> big(n, q.get_context());
    compute::future<compute::vector<int>::iterator> up = compute::copy_async(hp, hp + n, big.begin(), q);
    compute::command_queue q2(q.get_context(), compute::system::default_device());
    up.get_event().enqueue_wait(q2);
    int sum = 0;  // about 3 * 2^24: fits an int
    compute::reduce(big.begin(), big.end(), &sum, q2);
    up.wait();
    CHECK(up.get_event().status() == compute::event::complete);
    CHECK(up.get_event().duration<std::chrono::microseconds>().count() > 0);
    int expect = 0;
    for (size_t i = 0; i < n; ++i) expect += int(i % 7);
    CHECK(sum == expect);
    bcx_free_host(pinned);
  }
  compute::event never;  // never recorded: complete, and wait() returns
  never.wait();
  CHECK(never.status() == compute::event::complete);
}

static int run_all();

int main() {
  try {
    return run_all();
  } catch (const compute::program_build_failure &e) {
    std::printf("FAILED: program_build_failure\n%s\n", e.build_log().c_str());
  } catch (const std::exception &e) {
    std::printf("FAILED: exception %s\n", e.what());
  }
  return 1;
}

static int run_all() {
  compute::command_queue &q = compute::system::default_queue();
  readme_example();
  sort_cases(q);
  scan_cases(q);
  reduce_cases(q);
  transform_cases(q);
  reduce_by_key_cases(q);
  jit_cases(q);
  jit_large_cases(q);
  jit_staged_cases(q);
  zip_view_cases(q);
  transform_reduce_cases(q);
  scan_family_cases(q);
  comparator_sort_cases(q);
  compaction_cases(q);
  error_cases(q);
  async_cases(q);
  q.check_device_errors();
  std::printf("%s (%d failures)\n", g_failures ? "FAILED" : "OK", g_failures);
  return g_failures ? 1 : 0;
}
