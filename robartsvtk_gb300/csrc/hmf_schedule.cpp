// hmf_schedule.cpp -- adjoint schedules (see hmf_schedule.hpp).
//
// Fewest-forward-iterations schedule.  Costs count forward iterations.
//   R(l, f, h): reverse the l iterations t0 .. t1-1 (t1 = t0 + l) given x_t0
//     in a slot that stays held, f free slots, and x_t1 held in one more slot
//     (h = 1, released after the backward step of t1-1) or not held (h = 0).
//       l = 1:  h ? 0 : 1 (one forward iteration into a free slot), f >= 1 - h;
//       l > 1:  min over m in [1, l-1] with f >= (m >= 2 ? 2 : 1) of
//               m + R(l-m, f-1, h) + min(R(m, f-1+h, 1), R(m, f+h, 0)):
//               advance x_t0 to x_{t0+m} into a free slot, reverse the upper
//               part from there, then the lower part keeping x_{t0+m} as its
//               x_t1 or releasing it.
//     With enough slots every inner state is kept: R = l-1 (h = 1, f >= l-1)
//     or l (h = 0, f >= l), the least possible.
//   P(l, f): compute x_T from x_t0 (T = t0 + l) and reverse everything:
//       min over m in [1, l] with f >= (m >= 2 ? 2 : 1) of
//         m = l:  l + R(l, f-1, 1)     (x_T kept for the last backward step)
//         m < l:  m + P(l-m, f-1) + min(R(m, f-1, 1), R(m, f, 0)),
//     P = l when f >= l.  The schedule for S slots is P(T, S-1).
#include "hmf_schedule.hpp"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <map>
#include <mutex>

namespace hmfi {
namespace {

constexpr long long kInf = INT64_MAX / 4;

struct Dp {
  int T = 0, F = 0, W = 0;        // W = F + 2 columns (f + h may reach F + 1 in unreachable entries)
  std::vector<long long> r;       // [(l * W + f) * 2 + h]
  std::vector<int> rm;            // choice: m * 2 + (release x_{t0+m} for the lower part)
  std::vector<long long> p;       // [l * W + f]
  std::vector<int> pm;

  long long R(int l, int f, int h) const {
    if (f < 0) return kInf;
    if (h ? f >= l - 1 : f >= l) return h ? l - 1 : l;
    if (f >= W) f = W - 1;
    return r[((size_t)l * W + f) * 2 + h];
  }
  long long P(int l, int f) const {
    if (f < 0) return kInf;
    if (f >= l) return l;
    if (f >= W) f = W - 1;
    return p[(size_t)l * W + f];
  }

  void solve(int T_, int slots) {
    T = T_;
    F = slots - 1;
    W = std::min(F, T) + 2;
    r.assign((size_t)(T + 1) * W * 2, kInf);
    rm.assign(r.size(), 0);
    p.assign((size_t)(T + 1) * W, kInf);
    pm.assign(p.size(), 0);
    for (int l = 1; l <= T; ++l) {
      for (int f = 0; f < W; ++f) {
        for (int h = 0; h < 2; ++h) {
          if (h ? f >= l - 1 : f >= l) continue;  // closed form
          long long best = kInf;
          int choice = 0;
          if (l == 1) {
            best = (h || f >= 1) ? (h ? 0 : 1) : kInf;
          } else {
            for (int m = 1; m < l; ++m) {
              if (f < (m >= 2 ? 2 : 1)) break;
              const long long up = R(l - m, f - 1, h);
              if (up >= kInf) continue;
              const long long keep = R(m, f - 1 + h, 1), drop = R(m, f + h, 0);
              const long long lo = std::min(keep, drop);
              if (lo >= kInf) continue;
              const long long c = m + up + lo;
              if (c < best) best = c, choice = m * 2 + (drop < keep ? 1 : 0);
            }
          }
          r[((size_t)l * W + f) * 2 + h] = best;
          rm[((size_t)l * W + f) * 2 + h] = choice;
        }
        if (f >= l) continue;
        long long best = kInf;
        int choice = 0;
        for (int m = 1; m <= l; ++m) {
          if (f < (m >= 2 ? 2 : 1)) break;
          long long c;
          int drop = 0;
          if (m == l) {
            const long long rest = R(l, f - 1, 1);
            if (rest >= kInf) continue;
            c = l + rest;
          } else {
            const long long up = P(l - m, f - 1);
            if (up >= kInf) continue;
            const long long keep = R(m, f - 1, 1), dr = R(m, f, 0);
            const long long lo = std::min(keep, dr);
            if (lo >= kInf) continue;
            drop = dr < keep ? 1 : 0;
            c = m + up + lo;
          }
          if (c < best) best = c, choice = m * 2 + drop;
        }
        p[(size_t)l * W + f] = best;
        pm[(size_t)l * W + f] = choice;
      }
    }
  }
};

struct Emitter {
  const Dp& dp;
  std::vector<int> free;
  std::vector<AdjAction>& out;

  int pop() {
    const int s = free.back();
    free.pop_back();
    return s;
  }
  void fwd(int t, int a, int b) { out.push_back({kActForward, t, a, b}); }
  void bwd(int t, int a, int b) { out.push_back({kActBackward, t, a, b}); }

  // x_t0 (slot c0) -> x_{t0+m} in a slot taken from the free ones
  int advance(int t0, int m, int c0) {
    if (m == 1) {
      const int q = pop();
      fwd(t0, c0, q);
      return q;
    }
    int cur = pop(), other = pop();
    fwd(t0, c0, cur);
    for (int i = 1; i < m; ++i) {
      fwd(t0 + i, cur, other);
      std::swap(cur, other);
    }
    free.push_back(other);
    return cur;
  }

  // every state of t0 .. t0+l kept: x_{t0+l} is c1 if held, else computed
  void keep_all(int t0, int l, int c0, int c1, bool loss) {
    std::vector<int> s((size_t)l + 1);
    s[0] = c0;
    const int last = c1 >= 0 ? l - 1 : l;
    for (int i = 1; i <= last; ++i) {
      s[i] = pop();
      fwd(t0 + i - 1, s[i - 1], s[i]);
    }
    if (c1 >= 0) s[l] = c1;
    if (loss) out.push_back({kActLoss, t0 + l, s[l], -1});
    for (int i = l - 1; i >= 0; --i) {
      bwd(t0 + i, s[i], s[i + 1]);
      free.push_back(s[i + 1]);
    }
  }

  void reverse(int t0, int l, int c0, int c1) {
    const int f = (int)free.size(), h = c1 >= 0 ? 1 : 0;
    if (h ? f >= l - 1 : f >= l) return keep_all(t0, l, c0, c1, false);
    const int choice = dp.rm[((size_t)l * dp.W + std::min(f, dp.W - 1)) * 2 + h];
    const int m = choice / 2;
    const bool drop = choice & 1;
    const int cm = advance(t0, m, c0);
    reverse(t0 + m, l - m, cm, c1);
    if (drop) {
      free.push_back(cm);
      reverse(t0, m, c0, -1);
    } else {
      reverse(t0, m, c0, cm);
    }
  }

  void top(int t0, int l, int c0) {
    const int f = (int)free.size();
    if (f >= l) return keep_all(t0, l, c0, -1, true);
    const int choice = dp.pm[(size_t)l * dp.W + std::min(f, dp.W - 1)];
    const int m = choice / 2;
    const bool drop = choice & 1;
    const int cm = advance(t0, m, c0);
    if (m == l) {
      out.push_back({kActLoss, t0 + l, cm, -1});
      reverse(t0, l, c0, cm);
      return;
    }
    top(t0 + m, l - m, cm);
    if (drop) {
      free.push_back(cm);
      reverse(t0, m, c0, -1);
    } else {
      reverse(t0, m, c0, cm);
    }
  }
};

long long count_forward(const std::vector<AdjAction>& a) {
  long long n = 0;
  for (const auto& x : a) n += x.kind == kActForward;
  return n;
}

}  // namespace

AdjSchedule schedule_fixed(int T, int k) {
  AdjSchedule S;
  k = std::max(1, std::min(k, std::max(T, 1)));
  const int n_ckpt = std::max(1, (T + k - 1) / k);
  S.slots = n_ckpt + k;
  S.k = k;
  S.recomputed_segments = n_ckpt - 1;
  // C_m = m, S_j = n_ckpt + j - 1; state a + j of the segment from a in S_j
  auto src = [&](int t) {
    const int a = (t / k) * k;
    return t == a ? a / k : n_ckpt + (t - a) - 1;
  };
  auto dst = [&](int t) {
    const int a = (t / k) * k;
    if ((t + 1) % k == 0 && t + 1 < T) return (t + 1) / k;
    return n_ckpt + (t + 1 - a) - 1;
  };
  for (int t = 0; t < T; ++t) S.actions.push_back({kActForward, t, src(t), dst(t)});
  S.actions.push_back({kActLoss, T, T > 0 ? dst(T - 1) : 0, -1});
  const int a_last = T > 0 ? ((T - 1) / k) * k : 0;
  for (int a = a_last; a >= 0 && T > 0; a -= k) {
    const int b = std::min(a + k, T);
    if (a != a_last)
      for (int t = a; t + 2 <= b; ++t) S.actions.push_back({kActForward, t, src(t), dst(t)});
    for (int t = b - 1; t >= a; --t) S.actions.push_back({kActBackward, t, src(t), dst(t)});
  }
  S.forward = count_forward(S.actions);
  return S;
}

// The dynamic program costs about T^2 * min(S, T) / 3 steps (~20-30 ns each
// on a host core).  Beyond kDpMaxWork steps, checkpoints every k <= sqrt(T)
// iterations are used instead when they fit (about two forward passes, close
// to the optimum with that many slots); the dynamic program runs only when
// they do not.  Schedules are cached per (T, S): a training loop calls the
// adjoint with the same iteration count and memory budget again and again.
constexpr double kDpMaxWork = 5.0e7;

bool schedule_fewest_uncached(int T, int slots, AdjSchedule* out);

bool schedule_fewest(int T, int slots, AdjSchedule* out) {
  static std::mutex mu;
  static std::map<std::pair<int, int>, AdjSchedule> cache;
  {
    std::lock_guard<std::mutex> lock(mu);
    auto it = cache.find({T, slots});
    if (it != cache.end()) {
      *out = it->second;
      return true;
    }
  }
  if (!schedule_fewest_uncached(T, slots, out)) return false;
  std::lock_guard<std::mutex> lock(mu);
  if (cache.size() > 64) cache.clear();
  cache[{T, slots}] = *out;
  return true;
}

bool schedule_fewest_uncached(int T, int slots, AdjSchedule* out) {
  if (T < 0 || slots < 1) return false;
  if (T > 0 && slots < T + 1 && (double)T * T * std::min(slots, T) / 3.0 > kDpMaxWork) {
    for (int k = std::max(1, (int)std::ceil(std::sqrt((double)T))); k >= 1; --k)
      if ((T + k - 1) / k + k <= slots) {
        *out = schedule_fixed(T, k);
        return true;
      }
  }
  AdjSchedule S;
  if (T == 0) {
    S.slots = 1;
    S.actions.push_back({kActLoss, 0, 0, -1});
    *out = S;
    return true;
  }
  if (slots >= T + 1) {  // every state kept
    *out = schedule_fixed(T, T);
    return true;
  }
  Dp dp;
  dp.solve(T, slots);
  if (dp.P(T, slots - 1) >= kInf) return false;
  Emitter em{dp, {}, S.actions};
  for (int s = slots - 1; s >= 1; --s) em.free.push_back(s);  // pop() takes the lowest id first
  em.top(0, T, 0);
  S.slots = slots;
  S.forward = count_forward(S.actions);
  *out = S;
  return true;
}

long long schedule_fewest_cost(int T, int slots) {
  AdjSchedule sc;
  return schedule_fewest(T, slots, &sc) ? sc.forward : -1;
}

}  // namespace hmfi
