// Where the yielded items of a system go: the (t, y) stream the reference
// iterator produces, one item per accepted step (src/ivp.rs:214-238).
//
// Two layouts, chosen per launch:
// - packed (off != null): system i's items occupy [off[i], off[i+1]) of one
//   stream, CSR style.  The host fills off from a first pass's accepted
//   counts (an exclusive scan), so every system has exactly the room it
//   needs and nothing is wasted between systems;
// - slab (off == null): system i owns cap slots at i * cap.
// An item without a slot is never dropped silently: the kernel ends that
// system with BACON_CAPACITY_EXCEEDED before yielding it.
#pragma once

#include <cstdint>

namespace bacon {

// Slot of item k of system idx, or -1 when its buffer is full.
__device__ __forceinline__ int64_t traj_slot(const int64_t* off, int32_t cap, int64_t idx, int32_t k) {
  if (off != nullptr) {
    const int64_t b = off[idx];
    return (static_cast<int64_t>(k) < off[idx + 1] - b) ? b + k : -1;
  }
  return (k < cap) ? idx * cap + k : -1;
}

}  // namespace bacon
