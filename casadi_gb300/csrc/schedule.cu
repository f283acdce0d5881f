// Register-pressure scheduling of SX tapes (host code).
//
// CasADi orders an SXFunction's algorithm by a depth-first sort of the expression graph and
// then assigns work-vector slots to live values last-in first-out (SXFunction::init,
// casadi/core/sx_function.cpp:530-540 and 690-753): the work vector is as long as the largest
// number of values live at one point of THAT order. On the GPU each 32-instance tile keeps its work
// vector in shared memory, so its length decides how many warps an SM holds, and the sweeps
// are latency-bound: fewer live values means more warps in flight.
//
// The scheduler here is a greedy list scheduler over the value graph: among the instructions
// whose operands are available it takes the one that defines the fewest new live values net of
// the values it ends (its score is defines - frees), then the one whose oldest operand was
// defined first, then the earliest in the original order. Two kinds of edges constrain it:
// data dependences, and between consecutive users of each non-constant value (so the adjoint
// sums of every value keep their order, see schedule.cuh).
#include <algorithm>
#include <cstdio>
#include <queue>
#include <tuple>
#include <unordered_map>

#include "schedule.cuh"

namespace cgb {

namespace {

bool defines_value(unsigned op) { return op != D_OUTPUT && op != D_NOP; }

// Slots for the values in `order`: an operand's slot is freed at its last use, before the
// result is placed, so the result may take it (the sweeps read operands before writing the
// result); freed slots are reused last-in first-out. Returns the work-vector length.
int assign_slots(const std::vector<u64>& in, const std::vector<int>& order,
                 const std::vector<int>& dep0, const std::vector<int>& dep1,
                 std::vector<u64>& out) {
  const int n = static_cast<int>(order.size());
  std::vector<int> pos(n), last(n, -1), slot(n, -1), free_slots;
  for (int p = 0; p < n; ++p) pos[order[p]] = p;
  for (int k = 0; k < n; ++k) {
    if (dep0[k] >= 0) last[dep0[k]] = std::max(last[dep0[k]], pos[k]);
    if (dep1[k] >= 0) last[dep1[k]] = std::max(last[dep1[k]], pos[k]);
  }
  int n_slots = 0;
  out.resize(n);
  for (int p = 0; p < n; ++p) {
    const int k = order[p];
    const u64 w = in[k];
    const unsigned op = dec_op(w);
    for (int d : {dep0[k], dep1[k]})
      if (d >= 0 && last[d] == p) free_slots.push_back(slot[d]);
    if (defines_value(op)) {
      if (free_slots.empty()) {
        slot[k] = n_slots++;
      } else {
        slot[k] = free_slots.back();
        free_slots.pop_back();
      }
      if (last[k] < 0) free_slots.push_back(slot[k]);  // never read
    }
    switch (op) {
      case D_NOP:
        out[p] = w;
        break;
      case D_CONST:
      case D_INPUT:
        out[p] = enc(op, slot[k], dec_b(w), dec_c(w));
        break;
      case D_OUTPUT:
        out[p] = enc(op, dec_a(w), slot[dep0[k]], dec_c(w));
        break;
      default: {
        const int b = slot[dep0[k]];
        const int c = is_binary(op) ? slot[dep1[k] >= 0 ? dep1[k] : dep0[k]] : b;
        out[p] = enc(op, slot[k], b, c);
      }
    }
  }
  return n_slots;
}

}  // namespace

int schedule_code(const std::vector<u64>& in, std::vector<u64>& out, std::string& err) {
  const int n = static_cast<int>(in.size());
  out.clear();
  if (n == 0) return 0;
  // value graph: dep0/dep1 = defining instruction of each operand (-1: none)
  std::vector<int> dep0(n, -1), dep1(n, -1);
  std::vector<int> cur;  // slot -> defining instruction of its current value
  auto def_of = [&](unsigned slot, int k, int* d) {
    if (slot >= cur.size() || cur[slot] < 0) {
      char buf[128];
      std::snprintf(buf, sizeof(buf), "instruction %d reads slot %u before it is written", k, slot);
      err = buf;
      return false;
    }
    *d = cur[slot];
    return true;
  };
  for (int k = 0; k < n; ++k) {
    const u64 w = in[k];
    const unsigned op = dec_op(w);
    if (op == D_NOP) continue;
    if (op == D_OUTPUT) {
      if (!def_of(dec_b(w), k, &dep0[k])) return -1;
    } else if (op != D_CONST && op != D_INPUT) {
      if (!def_of(dec_b(w), k, &dep0[k])) return -1;
      if (is_binary(op)) {
        int d = -1;
        if (!def_of(dec_c(w), k, &d)) return -1;
        if (d != dep0[k]) dep1[k] = d;
      }
    }
    if (defines_value(op)) {
      const unsigned a = dec_a(w);
      if (a >= cur.size()) cur.resize(a + 1, -1);
      cur[a] = k;
    }
  }
  // users of each value, in original order (one entry per user instruction)
  std::vector<int> ucount(n, 0);
  for (int k = 0; k < n; ++k) {
    if (dep0[k] >= 0) ++ucount[dep0[k]];
    if (dep1[k] >= 0) ++ucount[dep1[k]];
  }
  std::vector<int> ustart(n + 1, 0);
  for (int k = 0; k < n; ++k) ustart[k + 1] = ustart[k] + ucount[k];
  std::vector<int> users(ustart[n]);
  {
    std::vector<int> fill(ustart.begin(), ustart.end() - 1);
    for (int k = 0; k < n; ++k) {
      if (dep0[k] >= 0) users[fill[dep0[k]]++] = k;
      if (dep1[k] >= 0) users[fill[dep1[k]]++] = k;
    }
  }
  // predecessor counts: data edges plus user-order edges (u_i -> u_{i+1} for each value).
  // Constants are exempt from the user order: the adjoint a constant's slot collects is
  // discarded (CONST has no operands to pass it to), so its summation order does not matter.
  std::vector<int> npred(n, 0);
  std::vector<std::vector<int>> succ(n);
  auto edge = [&](int p, int s) {
    succ[p].push_back(s);
    ++npred[s];
  };
  for (int k = 0; k < n; ++k) {
    if (dep0[k] >= 0) edge(dep0[k], k);
    if (dep1[k] >= 0) edge(dep1[k], k);
  }
  for (int d = 0; d < n; ++d) {
    if (dec_op(in[d]) == D_CONST) continue;
    for (int q = ustart[d] + 1; q < ustart[d + 1]; ++q) edge(users[q - 1], users[q]);
  }

  // priority of a ready instruction: (defines - frees, position of its oldest operand in the
  // new order, original position), smallest first. Taking the instruction whose operand has
  // waited longest ends long live ranges early.
  std::vector<int> remaining(ucount), newpos(n, -1);
  std::vector<char> done(n, 0);
  auto score = [&](int k) {
    int s = defines_value(dec_op(in[k])) ? 1 : 0;
    if (dep0[k] >= 0 && remaining[dep0[k]] == 1) --s;
    if (dep1[k] >= 0 && remaining[dep1[k]] == 1) --s;
    return s;
  };
  auto oldest = [&](int k) {
    int o = n;
    if (dep0[k] >= 0) o = std::min(o, newpos[dep0[k]]);
    if (dep1[k] >= 0) o = std::min(o, newpos[dep1[k]]);
    return o;
  };
  typedef std::tuple<int, int, int> Entry;
  std::priority_queue<Entry, std::vector<Entry>, std::greater<Entry>> heap;
  auto push = [&](int k) { heap.push(Entry(score(k), oldest(k), k)); };
  for (int k = 0; k < n; ++k)
    if (npred[k] == 0) push(k);
  std::vector<int> order;
  order.reserve(n);
  while (!heap.empty()) {
    const int k = std::get<2>(heap.top());
    heap.pop();
    if (done[k]) continue;  // an entry superseded by one with a lower score
    done[k] = 1;
    newpos[k] = static_cast<int>(order.size());
    order.push_back(k);
    for (int d : {dep0[k], dep1[k]}) {
      if (d < 0) continue;
      if (--remaining[d] == 1) {
        // the one user left now frees d: lower its score if it is waiting
        for (int q = ustart[d + 1] - 1; q >= ustart[d]; --q) {
          const int u = users[q];
          if (done[u]) continue;
          if (npred[u] == 0) push(u);
          break;
        }
      }
    }
    for (int s : succ[k])
      if (--npred[s] == 0) push(s);
  }
  if (static_cast<int>(order.size()) != n) {
    err = "tape has a dependence cycle";
    return -1;
  }
  // keep whichever order needs the shorter work vector
  std::vector<int> identity(n);
  for (int k = 0; k < n; ++k) identity[k] = k;
  std::vector<u64> alt;
  const int w_sched = assign_slots(in, order, dep0, dep1, out);
  const int w_orig = assign_slots(in, identity, dep0, dep1, alt);
  if (w_orig < w_sched) {
    out.swap(alt);
    return w_orig;
  }
  return w_sched;
}

int level_schedule(const std::vector<u64>& in, int width, int slot_cap, Levels& out,
                   std::string& err, bool ordered_users) {
  const int n = static_cast<int>(in.size());
  out = Levels();
  out.begin.push_back(0);
  if (width < 1) width = 1;
  // value graph (dep0/dep1: defining instruction of each operand) and recorded-partial indices
  std::vector<int> dep0(n, -1), dep1(n, -1), after(n, -1), pidx(n, 0);
  std::vector<int> cur;                      // slot -> defining instruction of its value
  std::unordered_map<long long, int> last_out;  // (output, nonzero) -> last OUTPUT writing it
  int np = 0;
  for (int k = 0; k < n; ++k) {
    const u64 w = in[k];
    const unsigned op = dec_op(w);
    pidx[k] = np;
    if (op == D_NOP) continue;
    auto def_of = [&](unsigned slot, int* d) {
      if (slot >= cur.size() || cur[slot] < 0) {
        char buf[128];
        std::snprintf(buf, sizeof(buf), "instruction %d reads slot %u before it is written", k,
                      slot);
        err = buf;
        return false;
      }
      *d = cur[slot];
      return true;
    };
    if (op == D_OUTPUT) {
      if (!def_of(dec_b(w), &dep0[k])) return -1;
      // two writes of one output nonzero keep their order
      const long long key = (static_cast<long long>(dec_a(w)) << 32) | dec_c(w);
      auto it = last_out.find(key);
      if (it != last_out.end()) {
        after[k] = it->second;
        it->second = k;
      } else {
        last_out.emplace(key, k);
      }
    } else if (op != D_CONST && op != D_INPUT) {
      if (!def_of(dec_b(w), &dep0[k])) return -1;
      if (is_binary(op)) {
        int d = -1;
        if (!def_of(dec_c(w), &d)) return -1;
        if (d != dep0[k]) dep1[k] = d;
      }
      const unsigned m = partial_mask(op);
      np += static_cast<int>((m & 1u) + ((m >> 1) & 1u));
    }
    if (defines_value(op)) {
      const unsigned a = dec_a(w);
      if (a >= cur.size()) cur.resize(a + 1, -1);
      cur[a] = k;
    }
  }
  // successors, predecessor counts, remaining uses
  std::vector<std::vector<int>> succ(n);
  std::vector<int> npred(n, 0), uses(n, 0);
  for (int k = 0; k < n; ++k)
    for (int d : {dep0[k], dep1[k], after[k]})
      if (d >= 0) {
        succ[d].push_back(k);
        ++npred[k];
      }
  for (int k = 0; k < n; ++k)
    for (int d : {dep0[k], dep1[k]})
      if (d >= 0) ++uses[d];
  if (ordered_users) {
    // consecutive users of each non-constant value in consecutive levels: the reverse sweep
    // then adds the contributions to every adjoint in the order of `in` (last user first)
    std::vector<int> last_user(n, -1);
    for (int k = 0; k < n; ++k)
      for (int d : {dep0[k], dep1[k]}) {
        if (d < 0 || dec_op(in[d]) == D_CONST) continue;
        if (last_user[d] >= 0 && last_user[d] != k) {
          succ[last_user[d]].push_back(k);
          ++npred[k];
        }
        last_user[d] = k;
      }
  }

  // Priority: position in `in` (the register-pressure order). The earliest ready instruction
  // of each level always runs -- that is the sequential order's own progress, which needs no
  // more slots than the order itself -- and later ready instructions fill the level only
  // while fewer than `slot_cap` values are live or a slot is free, so looking ahead for
  // parallel work never grows the work vector much past the cap.
  typedef int Entry;
  std::priority_queue<Entry, std::vector<Entry>, std::greater<Entry>> ready;
  for (int k = 0; k < n; ++k)
    if (dec_op(in[k]) != D_NOP && npred[k] == 0) ready.push(k);
  std::vector<int> slot(n, -1), free_slots;  // free_slots: usable in the current level
  int n_slots = 0, live = 0, placed = 0, total = 0;
  for (int k = 0; k < n; ++k) total += dec_op(in[k]) != D_NOP;
  std::vector<int> chosen, deferred, freed;
  const int max_deferred = 4 * width;
  while (placed < total) {
    chosen.clear();
    deferred.clear();
    while (!ready.empty() && static_cast<int>(chosen.size()) < width &&
           static_cast<int>(deferred.size()) < max_deferred) {
      const int k = ready.top();
      ready.pop();
      if (defines_value(dec_op(in[k]))) {
        if (!chosen.empty() && free_slots.empty() && live >= slot_cap) {
          deferred.push_back(k);
          continue;
        }
        if (free_slots.empty()) {
          slot[k] = n_slots++;
        } else {
          slot[k] = free_slots.back();
          free_slots.pop_back();
        }
        ++live;
      }
      chosen.push_back(k);
    }
    if (chosen.empty()) {
      err = "tape has a dependence cycle";
      return -1;
    }
    for (int k : deferred) ready.push(k);
    // emit the level
    freed.clear();
    for (int k : chosen) {
      const u64 w = in[k];
      const unsigned op = dec_op(w);
      switch (op) {
        case D_CONST:
        case D_INPUT:
          out.code.push_back(enc(op, slot[k], dec_b(w), dec_c(w)));
          break;
        case D_OUTPUT:
          out.code.push_back(enc(op, dec_a(w), slot[dep0[k]], dec_c(w)));
          break;
        default: {
          const int b = slot[dep0[k]];
          const int c = is_binary(op) ? slot[dep1[k] >= 0 ? dep1[k] : dep0[k]] : b;
          out.code.push_back(enc(op, slot[k], b, c));
        }
      }
      out.pidx.push_back(pidx[k]);
      out.src.push_back(k);
      for (int d : {dep0[k], dep1[k]})
        if (d >= 0 && --uses[d] == 0) freed.push_back(d);
      if (defines_value(op) && uses[k] == 0) freed.push_back(k);  // never read
    }
    out.begin.push_back(static_cast<int>(out.code.size()));
    placed += static_cast<int>(chosen.size());
    // slots of values whose last use was in this level are free from the next level on
    for (int d : freed) {
      free_slots.push_back(slot[d]);
      --live;
    }
    for (int k : chosen)
      for (int s : succ[k])
        if (--npred[s] == 0) ready.push(s);
  }
  out.sz_w = n_slots;
  return static_cast<int>(out.begin.size()) - 1;
}

}  // namespace cgb
