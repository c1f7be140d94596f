// wang.hpp -- host-side Wang et al. online checkpoint placement.
//
// Same schedule as the reference's DynamicCheckpointing::makeCheckpoint
// (topOpt/dynamicCheckpointing.cc:9-54) and WangCheckpointing::getForwardSolution
// / computeNewCheckpoints (topOpt/WangCheckpointing.cc:72-162): a list of
// checkpoints ordered newest first, each with a step, a level and a storage
// slot; when storage runs out, either the checkpoint after the reader is
// dropped (if its level is lower) or the newest one is replaced with its level
// raised by one.  Snapshots are device buffers indexed by slot; the caller
// supplies the three actions the reference's CheckpointingBase leaves virtual
// (advance, setSolverState, copyFromSolverState, checkpointingBase.hh:11-17).
//
// The list is kept in a node pool.  An erased node keeps its fields and links
// and freed nodes are reused oldest-first, so a restart point whose node is
// dropped while new checkpoints are placed still reads its original step and
// neighbour, as the reference's std::list iterator does in that case.
#pragma once

#include <climits>
#include <cstdint>
#include <deque>
#include <functional>
#include <stdexcept>
#include <vector>

namespace lbm {

class WangSchedule {
 public:
  struct Actions {
    std::function<int(void)> advance;               // one forward step of the solver
    std::function<int(int step, int slot)> restore; // solver state <- slot, time <- step
    std::function<int(int slot)> save;              // slot <- solver state
  };

  explicit WangSchedule(int nslots) : nslots_(nslots) { reset(); }

  void reset() {
    nodes_.clear();
    free_.clear();
    head_ = -1;
    reader_ = -1;
    avail_.clear();
    // the reference pushes storage[0..K-1] on a stack: slot K-1 is used first
    for (int i = 0; i < nslots_; ++i) avail_.push_back(i);
    recomputed_ = 0;
  }

  int64_t recomputed() const { return recomputed_; }

  // Static placement (StaticCheckpointing, topOpt/staticCheckpointing.cc:3-63):
  // the checkpoints this schedule computes for `nsteps` steps from an empty
  // list, oldest first; after plan_static, make_checkpoint_static keeps exactly
  // those states and the reverse sweep (get_forward_solution) is unchanged.
  void plan_static(int nsteps) {
    reset();
    compute_new_checkpoints(nsteps);
    plan_.clear();
    int tail = head_;
    while (tail >= 0 && nodes_[tail].next >= 0) tail = nodes_[tail].next;
    for (int id = tail; id >= 0; id = nodes_[id].prev) plan_.push_back({nodes_[id].step, nodes_[id].level});
    reset();
    plan_pos_ = 0;
  }

  // Static counterpart of make_checkpoint: the slot to copy state `index`
  // into, or -1 when the plan does not keep it.
  int make_checkpoint_static(int index) {
    if (plan_pos_ >= plan_.size() || plan_[plan_pos_].step != index) return -1;
    const int slot = pop_avail();
    push_front(index, plan_[plan_pos_].level, slot);
    ++plan_pos_;
    return slot;
  }

  // Place checkpoint `index`; returns the slot the caller must copy the state into.
  int make_checkpoint(int index) {
    if (head_ < 0) {
      int slot = pop_avail();
      reader_ = push_front(index, INT_MAX, slot);
      return slot;
    }
    if (!avail_.empty()) {
      int slot = pop_avail();
      reader_ = push_front(index, 0, slot);
      return slot;
    }
    int movable = nodes_[reader_].next;
    if (movable < 0) throw std::logic_error("checkpoint list exhausted");
    if (nodes_[movable].level < nodes_[reader_].level) {
      int slot = nodes_[movable].slot;
      push_front(index, 0, slot);
      erase(movable);
      return slot;
    }
    int r = head_;
    int level = nodes_[r].level + 1;
    int slot = nodes_[r].slot;
    push_front(index, level, slot);
    erase(r);
    reader_ = head_;
    return slot;
  }

  // Bring the state of step `index` into the solver (recomputing from the
  // nearest checkpoint and placing new ones), then release its checkpoint.
  int get_forward_solution(int index, const Actions& act) {
    int init = head_;
    if (init < 0) throw std::logic_error("no checkpoints");
    int rc;
    if (nodes_[init].step != index) {
      init = compute_new_checkpoints(index);
      int cur = nodes_[init].step;
      if ((rc = act.restore(cur, nodes_[init].slot))) return rc;
      init = nodes_[init].prev;
      for (;;) {
        if ((rc = act.advance())) return rc;
        ++cur;
        ++recomputed_;
        if (nodes_[init].step == cur) {
          if (nodes_[init].step == index) break;
          if ((rc = act.save(nodes_[init].slot))) return rc;
          init = nodes_[init].prev;
        }
      }
    } else {
      if ((rc = act.restore(index, nodes_[init].slot))) return rc;
    }
    avail_.push_back(nodes_[init].slot);
    erase(init);
    return 0;
  }

 private:
  struct Node {
    int step, level, slot, prev, next;
  };

  int pop_avail() {
    int s = avail_.back();
    avail_.pop_back();
    return s;
  }

  int alloc_node() {
    if (!free_.empty()) {
      int id = free_.front();
      free_.pop_front();
      return id;
    }
    nodes_.push_back(Node{0, 0, 0, -1, -1});
    return (int)nodes_.size() - 1;
  }

  int push_front(int step, int level, int slot) {
    int id = alloc_node();
    nodes_[id] = Node{step, level, slot, -1, head_};
    if (head_ >= 0) nodes_[head_].prev = id;
    head_ = id;
    return id;
  }

  void erase(int id) {
    int p = nodes_[id].prev, n = nodes_[id].next;
    if (p >= 0)
      nodes_[p].next = n;
    else
      head_ = n;
    if (n >= 0) nodes_[n].prev = p;
    free_.push_back(id);
  }

  int compute_new_checkpoints(int index) {
    if (head_ < 0) push_front(0, INT_MAX, pop_avail());
    int start = head_, reader = head_;
    int init_step = nodes_[start].step, nsteps = index - init_step;
    for (int ii = init_step; ii < init_step + nsteps; ++ii) {
      if (!avail_.empty()) {
        push_front(ii + 1, 0, pop_avail());
        reader = head_;
        continue;
      }
      int movable = nodes_[reader].next;
      if (nodes_[movable].level < nodes_[reader].level) {
        push_front(ii + 1, 0, nodes_[movable].slot);
        erase(movable);
      } else {
        reader = head_;
        int level = nodes_[reader].level + 1;
        push_front(ii + 1, level, nodes_[reader].slot);
        erase(reader);
        reader = head_;
      }
    }
    return start;
  }

  struct Planned {
    int step, level;
  };
  std::vector<Planned> plan_;
  size_t plan_pos_ = 0;

  int nslots_;
  std::vector<Node> nodes_;
  std::deque<int> free_;
  std::vector<int> avail_;
  int head_ = -1, reader_ = -1;
  int64_t recomputed_ = 0;
};

}  // namespace lbm
