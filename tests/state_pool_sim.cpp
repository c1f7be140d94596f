// Host simulation of the checkpointed gradient's buffer traffic: the Wang
// schedule (wang.hpp) driving the zero-copy StatePool (state_pool.hpp) the
// way lbm_gradient does, with every buffer holding the time step whose state
// it contains instead of a lattice.  Checks that each reverse step t sees the
// state of step t, that no time step writes over its own input or a live
// checkpoint, and counts the copies the pool asked for.
//
//   state_pool_sim NSTEPS NSNAP [static] -> prints "ok <copies> <recomputed>" or "FAIL ..."
#include <cstdio>
#include <cstdlib>
#include <stdexcept>
#include <vector>

#include "state_pool.hpp"
#include "wang.hpp"

using lbm::StatePool;
using lbm::WangSchedule;

int main(int argc, char** argv) {
  if (argc != 3 && argc != 4) return 2;
  const int nsteps = std::atoi(argv[1]), nsnap = std::atoi(argv[2]);
  const bool planned = argc == 4;
  std::vector<int> content(nsnap + 2, -100);   // buffer -> step held
  std::vector<int> slot_step(nsnap, -1);       // slot -> checkpointed step
  StatePool pool;
  pool.reset(nsnap, 0);
  WangSchedule ws(nsnap);
  if (planned) ws.plan_static(nsteps);
  auto place = [&](int index) { return planned ? ws.make_checkpoint_static(index) : ws.make_checkpoint(index); };
  long copies = 0;
  int t = 0;
  char err[256] = {0};

  auto check_write = [&](int out) {
    if (out == pool.current()) throw std::logic_error("time step writes its own input");
    for (int k = 0; k < nsnap; ++k)
      if (slot_step[k] >= 0 && pool.slot_buffer(k) == out)
        throw std::logic_error("time step writes a live checkpoint");
  };
  auto advance = [&]() {
    const int out = pool.scratch();
    check_write(out);
    if (content[pool.current()] != t) throw std::logic_error("input is not the current state");
    content[out] = t + 1;
    pool.set_current(out);
    ++t;
  };
  auto save = [&](int slot) {
    if (slot < 0) return;   // not kept by the static plan
    const int dst = pool.save(slot);
    if (dst >= 0) {
      ++copies;
      content[dst] = content[pool.current()];
    }
    slot_step[slot] = t;
    if (content[pool.slot_buffer(slot)] != t) throw std::logic_error("slot does not hold its step");
  };
  try {
    {
      const int out = pool.scratch();
      content[out] = 0;
      pool.set_current(out);
    }
    save(place(0));
    for (int s = 0; s < nsteps; ++s) {
      advance();
      save(place(s + 1));
    }
    WangSchedule::Actions act;
    act.advance = [&]() {
      advance();
      return 0;
    };
    act.restore = [&](int step, int slot) {
      if (slot_step[slot] != step) throw std::logic_error("restore of a slot that holds another step");
      pool.restore(slot);
      if (content[pool.current()] != step) throw std::logic_error("restored buffer holds another step");
      t = step;
      return 0;
    };
    act.save = [&](int slot) {
      save(slot);
      return 0;
    };
    for (int s = nsteps; s >= 1; --s) {
      ws.get_forward_solution(s, act);
      if (t != s || content[pool.current()] != s) {
        std::snprintf(err, sizeof(err), "reverse step %d saw the state of step %d", s,
                      content[pool.current()]);
        throw std::logic_error(err);
      }
    }
  } catch (const std::exception& e) {
    std::printf("FAIL %s\n", e.what());
    return 1;
  }
  std::printf("ok %ld %lld\n", copies, (long long)ws.recomputed());
  return 0;
}
