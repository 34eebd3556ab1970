// Host check of elx::BatchGate (elastic_gb300/csrc/elx_gate.h), the solve
// server's gate on block-solve batches; built and run by test_host_gate.py.
//   1. no small requests: all workers run batches at once;
//   2. a small request present: never more than one batch at a time;
//   3. small requests coming and going while workers run: every batch ends
//      (no lost wake-up), and the gate ends empty;
//   4. workers held back by a small request resume when it leaves.
#include <atomic>
#include <chrono>
#include <cstdio>
#include <thread>
#include <vector>

#include "elx_gate.h"

using Clock = std::chrono::steady_clock;

static int failures = 0;
#define CHECK(cond, ...)                  \
  do {                                    \
    if (!(cond)) {                        \
      std::printf("FAIL: " __VA_ARGS__);  \
      std::printf("\n");                  \
      failures++;                         \
    }                                     \
  } while (0)

static void sleep_us(int us) { std::this_thread::sleep_for(std::chrono::microseconds(us)); }

// Workers each run `batches` batches of `work_us`; returns the largest number
// of batches seen inside the gate at once.
static int run_workers(elx::BatchGate &g, int workers, int batches, int work_us,
                       std::atomic<int> &inside, std::atomic<int> &done) {
  std::atomic<int> peak{0};
  std::vector<std::thread> t;
  for (int w = 0; w < workers; w++)
    t.emplace_back([&] {
      for (int b = 0; b < batches; b++) {
        g.enter();
        const int now = ++inside;
        int p = peak.load();
        while (now > p && !peak.compare_exchange_weak(p, now)) {
        }
        sleep_us(work_us);
        --inside;
        g.leave();
        ++done;
      }
    });
  for (auto &x : t) x.join();
  return peak.load();
}

int main() {
  {  // 1. all workers at once: each waits inside until all three are in
    elx::BatchGate g(3);
    std::atomic<int> in{0};
    std::atomic<bool> all{false};
    std::vector<std::thread> t;
    for (int w = 0; w < 3; w++)
      t.emplace_back([&] {
        g.enter();
        ++in;
        const auto end = Clock::now() + std::chrono::seconds(5);
        while (in.load() < 3 && Clock::now() < end) sleep_us(100);
        if (in.load() == 3) all = true;
        g.leave();
      });
    for (auto &x : t) x.join();
    CHECK(all.load(), "three workers could not be inside the gate together");
    CHECK(g.running() == 0, "gate not empty after case 1");
  }
  {  // 2. one at a time while a small request is present
    elx::BatchGate g(4);
    g.small(1);
    std::atomic<int> in{0}, done{0};
    const int peak = run_workers(g, 4, 40, 200, in, done);
    CHECK(peak == 1, "%d batches at once with a small request present", peak);
    CHECK(done.load() == 160, "case 2: %d of 160 batches", done.load());
    g.small(-1);
    CHECK(g.running() == 0 && g.small_count() == 0, "gate not empty after case 2");
  }
  {  // 3. small requests coming and going: no batch is lost
    elx::BatchGate g(3);
    std::atomic<bool> stop{false};
    std::thread toggler([&] {
      while (!stop.load()) {
        g.small(1);
        sleep_us(150);
        g.small(1);
        sleep_us(50);
        g.small(-1);
        g.small(-1);
        sleep_us(120);
      }
    });
    std::atomic<int> in{0}, done{0};
    const auto t0 = Clock::now();
    run_workers(g, 3, 300, 30, in, done);
    stop = true;
    toggler.join();
    const double secs = std::chrono::duration<double>(Clock::now() - t0).count();
    CHECK(done.load() == 900, "case 3: %d of 900 batches", done.load());
    CHECK(secs < 60.0, "case 3 took %.1f s", secs);
    CHECK(g.running() == 0 && g.small_count() == 0, "gate not empty after case 3");
  }
  {  // 4. held back by a small request, released when it leaves
    elx::BatchGate g(2);
    g.enter();  // a running batch
    g.small(1);
    std::atomic<int> entered{0};
    std::thread w([&] {
      g.enter();
      ++entered;
      g.leave();
    });
    sleep_us(20000);
    CHECK(entered.load() == 0, "a second batch entered while a small request was present");
    g.small(-1);  // the limit goes back to 2: the waiting batch enters
    const auto end = Clock::now() + std::chrono::seconds(5);
    while (entered.load() == 0 && Clock::now() < end) sleep_us(100);
    CHECK(entered.load() == 1, "the waiting batch did not enter after the small request left");
    g.leave();
    w.join();
    CHECK(g.running() == 0, "gate not empty after case 4");
  }
  if (failures == 0) std::printf("gate_check: ok\n");
  return failures == 0 ? 0 : 1;
}
