// state_pool.hpp -- zero-copy checkpoint storage for the checkpointed gradient.
//
// The reference copies the solver's distributions into a checkpoint slot after
// each forward step and back before each reverse step
// (topOpt/LBCheckpointing.cc:50-66: setSolverState -> LBSolver::setDistributions,
// copyFromSolverState -> VecCopy of the distributions).  On the device those copies
// cost as much HBM traffic as the time steps themselves.  Here the current
// state and the K checkpoint slots are labels on one pool of K+2 equal
// buffers: a time step writes into a buffer that holds nothing live, a save
// re-labels the current buffer as the slot's, and a restore makes the slot's
// buffer current.  Nothing is copied except in the one case a save would make
// two slots share a buffer (a save right after a restore, which the online
// schedule never issues), where the caller copies.
#ifndef LBM_STATE_POOL_HPP
#define LBM_STATE_POOL_HPP

#include <stdexcept>
#include <vector>

namespace lbm {

class StatePool {
 public:
  // Buffers 0 and 1 are the solver's two state buffers, 2 .. K+1 the slots'
  // initial buffers; `cur` (0 or 1) holds the current state.
  void reset(int nslots, int cur) {
    slot_buf_.resize(nslots);
    holder_.assign(nslots + 2, -1);
    for (int k = 0; k < nslots; ++k) {
      slot_buf_[k] = k + 2;
      holder_[k + 2] = k;
    }
    cur_ = cur;
  }
  int buffers() const { return (int)holder_.size(); }
  int current() const { return cur_; }
  int slot_buffer(int slot) const { return slot_buf_.at(slot); }

  // A buffer a time step may write: neither the current state nor a slot's.
  // At most K buffers are held by slots, so one of the K+2 is always free.
  int scratch() const {
    for (int b = 0; b < (int)holder_.size(); ++b)
      if (b != cur_ && holder_[b] < 0) return b;
    throw std::logic_error("state pool: no free buffer");
  }
  void set_current(int b) { cur_ = b; }

  // Label the current state as `slot`'s checkpoint.  Returns -1 when that
  // needed no copy, else the buffer the caller must copy the current state
  // into (the slot keeps its own buffer).
  int save(int slot) {
    const int old = slot_buf_.at(slot);
    if (old == cur_) return -1;
    if (holder_[cur_] >= 0) return old;   // current buffer is another slot's
    holder_[old] = -1;
    holder_[cur_] = slot;
    slot_buf_[slot] = cur_;
    return -1;
  }
  // Make `slot`'s checkpoint the current state (it stays the slot's too).
  void restore(int slot) { cur_ = slot_buf_.at(slot); }

 private:
  std::vector<int> slot_buf_;   // slot -> buffer
  std::vector<int> holder_;     // buffer -> slot, or -1
  int cur_ = 0;
};

}  // namespace lbm

#endif  // LBM_STATE_POOL_HPP
