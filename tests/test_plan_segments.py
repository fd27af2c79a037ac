"""Host planning of the exact chain in segments (triplelens_gb300/csrc/plan.h)
without a GPU: the header compiles alone with g++, and on random sets of
curve lengths (including curves shorter than the number of segments) every
point is listed exactly once, each curve's segments are consecutive shares
in order with the curve as their chain, and the counts and offsets agree.
The seeds of a segmented chain equal one unbroken chain only if these hold
(the GPU tests check the seeds themselves).  The same header holds the
autotuner's choice among its timed candidates, tested here on set timings,
and the object batcher's gathering of concurrent callers, run here in threads
with emulated lens set-ups."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r"""
#include <cstdio>
#include <cstdlib>
#include <set>
#include "plan.h"

struct Job { int32_t traj, first, count, chain; };

int main() {
  unsigned seed = 12345u;
  auto rnd = [&]() { seed = seed * 1103515245u + 12345u; return (seed >> 8) & 0xffffff; };
  for (int trial = 0; trial < 300; trial++) {
    const int nseg = 1 + (int)(rnd() % 12);
    const int nc = 1 + (int)(rnd() % 20);
    std::vector<int64_t> base(nc);
    std::vector<uint32_t> n(nc);
    int64_t b = 0;
    for (int i = 0; i < nc; i++) {
      n[i] = (uint32_t)(rnd() % 60);          // 1..60 points, often fewer than nseg
      base[i] = b;
      b += (int64_t)n[i] + 1;
    }
    std::vector<Job> jobs;
    std::vector<int32_t> list;
    std::vector<unsigned> count;
    std::vector<int> job0, off;
    tl::plan_segments(nseg, nc, base.data(), n.data(), &jobs, &list, &count, &job0, &off);
    if ((int64_t)list.size() != b) { printf("FAIL total %zu %lld\n", list.size(), (long long)b); return 1; }
    std::set<int32_t> seen(list.begin(), list.end());
    if ((int64_t)seen.size() != b) { printf("FAIL duplicates\n"); return 1; }
    if (job0[0] != 0 || off[0] != 0 || job0[nseg] != (int)jobs.size() || off[nseg] != (int)list.size()) {
      printf("FAIL ends\n"); return 1;
    }
    std::vector<long> next(nc, 0);           // next point expected per curve
    for (int s = 0; s < nseg; s++) {
      if (count[s] != (unsigned)(off[s + 1] - off[s])) { printf("FAIL count\n"); return 1; }
      int pos = off[s], prev = -1;
      for (int q = job0[s]; q < job0[s + 1]; q++) {
        const Job& j = jobs[q];
        if (j.chain != j.traj || j.traj <= prev || j.count <= 0) { printf("FAIL job\n"); return 1; }
        prev = j.traj;
        if (j.first != next[j.traj]) { printf("FAIL order\n"); return 1; }
        for (int k = 0; k < j.count; k++)
          if (list[pos++] != (int32_t)(base[j.traj] + j.first + k)) { printf("FAIL list\n"); return 1; }
        next[j.traj] = (long)j.first + j.count;
      }
      if (pos != off[s + 1]) { printf("FAIL offsets\n"); return 1; }
    }
    for (int i = 0; i < nc; i++)
      if (next[i] != (long)n[i] + 1) { printf("FAIL coverage\n"); return 1; }
  }
  printf("OK\n");
  return 0;
}
"""


PICK = r"""
#include <cstdio>
#include "plan.h"

static int fails = 0;
static void check(const char* what, std::initializer_list<float> t, int want) {
  std::vector<float> v(t);
  const int got = tl::pick_candidate(v.data(), (int)v.size(), 0.05f);
  if (got != want) { printf("FAIL %s: got %d want %d\n", what, got, want); fails++; }
}

int main() {
  check("default fastest", {100, 120, 130, 110, 140}, 0);
  check("within the margin", {100, 96, 99, 97, 98}, 0);
  check("exactly 5 % faster stays", {100, 95, 120, 120, 120}, 0);
  check("clearly faster wins", {100, 120, 80, 120, 120}, 2);
  // the fastest wins, not the first candidate past the margin
  check("fastest of several", {100, 94, 92, 120, 120}, 2);
  check("failed default", {-1, 120, 110, 130, 140}, 2);
  check("failed candidate ignored", {100, -1, 0, 99, 98}, 0);
  check("nothing ran", {-1, -1, -1, -1, -1}, 0);
  if (fails) return 1;
  printf("OK\n");
  return 0;
}
"""


GATHER = r"""
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <mutex>
#include <thread>
#include <vector>
#include "plan.h"

// the object batcher's structure (lcirs_abi.cu runBatched): requests queue,
// the first caller with no batch running leads, gathers, runs the batch
struct Sim {
  std::mutex mu;
  std::condition_variable cv;
  uint64_t arrivals = 0;
  std::vector<int*> pending;
  bool running = false;
  std::vector<size_t> batches;
  std::atomic<int> fresh{0}, constructing{0};

  void construct(int ms) {
    fresh++;
    constructing++;
    std::this_thread::sleep_for(std::chrono::milliseconds(ms));   // lens set-up
    constructing--;
  }
  void call(int run_ms) {
    int done = 0;
    std::unique_lock<std::mutex> lk(mu);
    fresh--;
    pending.push_back(&done);
    arrivals++;
    cv.notify_all();
    while (!done) {
      if (!running) {
        running = true;
        tl::gather_callers(lk, cv, arrivals, fresh, constructing);
        std::vector<int*> mine;
        mine.swap(pending);
        batches.push_back(mine.size());
        lk.unlock();
        std::this_thread::sleep_for(std::chrono::milliseconds(run_ms));   // the batch
        lk.lock();
        for (int* d : mine) *d = 1;
        running = false;
        cv.notify_all();
      } else {
        cv.wait(lk);
      }
    }
  }
};

int main() {
  using clk = std::chrono::steady_clock;
  // 152 objects created and called from a pool of threads, the first
  // object's set-up ending 10 ms before the others': one batch
  for (int rep = 0; rep < 3; rep++) {
    Sim s;
    std::vector<std::thread> th;
    std::atomic<int> ready{0};   // every thread exists before any set-up starts
    for (int k = 0; k < 152; k++)
      th.emplace_back([&s, &ready, k] {
        ready++;
        while (ready.load() < 152) std::this_thread::yield();
        s.construct(k == 0 ? 22 : 32);
        s.call(20);
      });
    for (auto& t : th) t.join();
    if (s.batches.size() != 1 || s.batches[0] != 152) {
      printf("FAIL pool: %zu batches, first %zu\n", s.batches.size(), s.batches[0]);
      return 1;
    }
  }
  // a lone caller waits one short gap, not the cap
  {
    Sim s;
    s.construct(1);
    const auto t0 = clk::now();
    s.call(0);
    const double ms = std::chrono::duration<double, std::milli>(clk::now() - t0).count();
    if (ms > 100.0) { printf("FAIL lone caller waited %.1f ms\n", ms); return 1; }
  }
  // a constructor that does not end soon: the cap closes the gathering
  {
    Sim s;
    std::thread slow([&s] { s.construct(1500); });
    std::this_thread::sleep_for(std::chrono::milliseconds(5));
    s.construct(1);
    const auto t0 = clk::now();
    s.call(0);
    const double ms = std::chrono::duration<double, std::milli>(clk::now() - t0).count();
    slow.join();
    if (ms < 250.0 || ms > 1000.0) { printf("FAIL cap: %.1f ms\n", ms); return 1; }
  }
  printf("OK\n");
  return 0;
}
"""


def _compile_and_run(tmp_path, name, program):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("no g++")
    src = tmp_path / (name + ".cc")
    src.write_text(program)
    exe = tmp_path / name
    r = subprocess.run([gxx, "-std=c++17", "-O1", "-pthread", "-I",
                        os.path.join(ROOT, "triplelens_gb300", "csrc"), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and r.stdout.strip() == "OK", r.stdout + r.stderr


def test_plan_segments_covers_every_point_once_in_chain_order(tmp_path):
    _compile_and_run(tmp_path, "plan_test", PROGRAM)


def test_autotuner_keeps_the_default_unless_the_fastest_beats_it_by_5_percent(tmp_path):
    """tlb_autotune's choice among its five fill-stage candidates
    (triplelens_gb300/csrc/batch_abi.cu) through tl::pick_candidate."""
    _compile_and_run(tmp_path, "pick_test", PICK)


def test_batcher_gathers_callers_whose_constructors_are_still_running(tmp_path):
    """The object batcher's gathering (tl::gather_callers, used by
    lcirs_abi.cu) in threads on the CPU: 152 callers whose first object's
    set-up ends 10 ms before the others' form one batch (counting objects
    only after their constructor split them 1 + 151); a lone caller waits
    a short gap; a constructor that does not end is cut off by the 300 ms
    cap."""
    _compile_and_run(tmp_path, "gather_test", GATHER)
