// hmf_schedule.hpp -- the order in which the adjoint runs forward iterations
// and backward steps over a bounded pool of state slots.
//
// A state slot holds one forward state x_t.  A forward iteration reads x_t
// from one slot and writes x_{t+1} into another (never in place: the flow
// kernel's windows read halos that neighbouring windows write), and the
// backward step of iteration t reads x_t and x_{t+1} from two slots.  With
// T + 1 slots every state is kept and each iteration runs forward once; with
// fewer, states are recomputed from kept ones.  Two schedules:
//
//  * fixed interval k: x_t kept for t a multiple of k (checkpoint slots),
//    the states of one segment recomputed into k segment slots when its
//    backward pass begins (k = T keeps every state);
//  * fewest forward iterations for a given number of slots S: a
//    revolve-style recursion (after Griewank's binomial checkpointing,
//    "Achieving logarithmic growth of temporal and spatial complexity in
//    reverse automatic differentiation", 1992) restated for this slot model
//    and solved by dynamic programming over (iterations left, free slots,
//    whether x_{t1} is held).  Advancing m >= 2 iterations without keeping
//    the states in between alternates between two free slots.
#pragma once

#include <vector>

namespace hmfi {

enum AdjActionKind { kActForward = 0, kActLoss = 1, kActBackward = 2 };

struct AdjAction {
  int kind;  // AdjActionKind
  int t;     // iteration (forward: x_t -> x_{t+1}; backward: reverse of iteration t)
  int a;     // forward: slot of x_t; loss: slot of x_T; backward: slot of x_t
  int b;     // forward: slot written with x_{t+1}; backward: slot of x_{t+1}
};

struct AdjSchedule {
  int slots = 0;              // state slots used (ids 0..slots-1; x_0 in slot 0)
  int k = 0;                  // checkpoint interval of a fixed-interval schedule, 0 otherwise
  int recomputed_segments = 0;
  long long forward = 0;      // forward iterations run, first pass included
  std::vector<AdjAction> actions;
};

// Fixed interval k (1 <= k <= T): ceil(T/k) checkpoint slots + k segment slots.
AdjSchedule schedule_fixed(int T, int k);

// Fewest forward iterations with at most `slots` state slots; false when no
// schedule exists (T >= 2 needs at least 3 slots).  For long runs
// (T^2 * min(slots, T) / 3 above 5e7) checkpoints every k <= sqrt(T)
// iterations are used instead when they fit.  Cached per (T, slots).
bool schedule_fewest(int T, int slots, AdjSchedule* out);

// Forward iterations of schedule_fewest(T, slots), -1 when infeasible.
long long schedule_fewest_cost(int T, int slots);

}  // namespace hmfi
