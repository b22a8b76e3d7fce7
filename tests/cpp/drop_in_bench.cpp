// Throughput of the drop-in boost::compute calls whose kernels are generated
// at run time, measured the way a reference caller reaches them:
//   * transform with the lambda alpha * _1 + _2 (perf/perf_saxpy.cpp:50-56)
//     over 2^28 float32 x, y ~ U[-1, 1] into a separate result;
//   * inclusive_scan and exclusive_scan with a BOOST_COMPUTE_FUNCTION adder
//     over 2^30 int32 in [0, 100);
//   * accumulate with the same user function over the same 2^30 int32.
// Each call is timed with events around it on the queue (device time), after
// warm-up calls (the first call compiles the kernel and fills the program
// cache); inputs are larger than L2.  Results are checked: saxpy bit for bit
// against fmaf on the host, the scans against the host's exact prefix sums
// (mod 2^32) on the first 2^24 elements and at sampled positions, the
// accumulate against the exact sum.  Prints one JSON object.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>

#include <boost/compute.hpp>

namespace compute = boost::compute;
using compute::_1;
using compute::_2;

template <class F>
static double time_ms(compute::command_queue &q, int warmup, int steps, F f) {
  for (int i = 0; i < warmup; ++i) f();
  q.finish();
  double total = 0.0;
  for (int i = 0; i < steps; ++i) {
    compute::event e = compute::event::around(q, [&](compute::command_queue &) { f(); });
    total += e.duration<std::chrono::duration<double, std::milli>>().count();
  }
  return total / steps;
}

int main(int argc, char **argv) {
  const int steps = argc > 1 ? std::atoi(argv[1]) : 5;
  const size_t n_saxpy = argc > 2 ? std::strtoull(argv[2], nullptr, 0) : (size_t(1) << 28);
  const size_t n_scan = argc > 3 ? std::strtoull(argv[3], nullptr, 0) : (size_t(1) << 30);
  compute::command_queue &q = compute::system::default_queue();
  bool ok = true;

  // ---- saxpy through the lambda -------------------------------------------
  double saxpy_ms = 0.0;
  {
    std::vector<float> hx(n_saxpy), hy(n_saxpy);
    std::mt19937 gen(20261203);
    std::uniform_real_distribution<float> u(-1.f, 1.f);
    for (size_t i = 0; i < n_saxpy; ++i) {
      hx[i] = u(gen);
      hy[i] = u(gen);
    }
    compute::vector<float> x(hx.begin(), hx.end(), q), y(hy.begin(), hy.end(), q), r(n_saxpy, q.get_context());
    const float alpha = 2.5f;
    saxpy_ms = time_ms(q, 3, steps, [&] { compute::transform(x.begin(), x.end(), y.begin(), r.begin(), alpha * _1 + _2, q); });
    std::vector<float> hr(n_saxpy);
    compute::copy(r.begin(), r.end(), hr.begin(), q);
    for (size_t i = 0; i < n_saxpy; i += 997)
      if (hr[i] != std::fmaf(alpha, hx[i], hy[i])) {
        ok = false;
        break;
      }
  }

  // ---- user-function scans and accumulate -----------------------------------
  double inc_ms = 0.0, exc_ms = 0.0, acc_ms = 0.0;
  {
    BOOST_COMPUTE_FUNCTION(int, add_u, (int a, int b), { return (int)((unsigned)a + (unsigned)b); });
    std::vector<int> ha(n_scan);
    std::mt19937 gen(7);
    unsigned long long exact = 0;
    for (size_t i = 0; i < n_scan; ++i) {
      ha[i] = int(gen() % 100u);
      exact += unsigned(ha[i]);
    }
    compute::vector<int> a(ha.begin(), ha.end(), q), out(n_scan, q.get_context());
    inc_ms = time_ms(q, 3, steps, [&] { compute::inclusive_scan(a.begin(), a.end(), out.begin(), add_u, q); });
    const size_t head = n_scan < (size_t(1) << 24) ? n_scan : (size_t(1) << 24);
    std::vector<int> ho(head);
    compute::copy(out.begin(), out.begin() + std::ptrdiff_t(head), ho.begin(), q);
    unsigned run = 0;
    for (size_t i = 0; i < head; ++i) {
      run += unsigned(ha[i]);
      if (unsigned(ho[i]) != run) {
        ok = false;
        break;
      }
    }
    int last = 0;
    compute::copy(out.end() - 1, out.end(), &last, q);
    if (unsigned(last) != unsigned(exact)) ok = false;
    exc_ms = time_ms(q, 3, steps, [&] { compute::exclusive_scan(a.begin(), a.end(), out.begin(), 5, add_u, q); });
    compute::copy(out.end() - 1, out.end(), &last, q);
    if (unsigned(last) != unsigned(exact - unsigned(ha[n_scan - 1]) + 5u)) ok = false;
    int sum = 0;
    acc_ms = time_ms(q, 3, steps, [&] { sum = compute::accumulate(a.begin(), a.end(), 0, add_u, q); });
    if (unsigned(sum) != unsigned(exact)) ok = false;
  }
  q.check_device_errors();
  std::printf(
      "{\"saxpy_lambda_f32\": {\"n\": %zu, \"ms\": %.4f, \"GB/s\": %.1f, \"bytes_per_elem\": 12, "
      "\"path\": \"transform(x, y, r, alpha * _1 + _2)\"}, "
      "\"user_function_inclusive_scan_i32\": {\"n\": %zu, \"ms\": %.4f, \"GB/s\": %.1f, \"bytes_per_elem\": 8}, "
      "\"user_function_exclusive_scan_i32\": {\"n\": %zu, \"ms\": %.4f, \"GB/s\": %.1f, \"bytes_per_elem\": 8}, "
      "\"user_function_accumulate_i32\": {\"n\": %zu, \"ms\": %.4f, \"GB/s\": %.1f, \"bytes_per_elem\": 4, "
      "\"note\": \"includes the blocking read of the result\"}, \"checked\": %s}\n",
      n_saxpy, saxpy_ms, 12.0 * n_saxpy / saxpy_ms / 1e6, n_scan, inc_ms, 8.0 * n_scan / inc_ms / 1e6, n_scan, exc_ms,
      8.0 * n_scan / exc_ms / 1e6, n_scan, acc_ms, 4.0 * n_scan / acc_ms / 1e6, ok ? "true" : "false");
  return ok ? 0 : 1;
}
