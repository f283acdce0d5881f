// Host-side instruction scheduling of an encoded tape for the GPU sweeps.
#pragma once
#include <string>
#include <vector>

#include "device_ops.cuh"

namespace cgb {

// Reorders an encoded tape (device opcodes, the reference's work-vector slots) so fewer values
// are live at once, and reassigns slots; returns the new work-vector length, or -1 with `err`
// set when the tape reads a slot before writing it.
//
// Every instruction still computes the same operation on the same operand values, so value,
// recorded-partial and tangent results are unchanged bit for bit. The users of each value keep
// their relative order, so the reverse sweep adds the contributions to each adjoint in the
// same sequence as the original order: adjoint results are unchanged bit for bit as well.
int schedule_code(const std::vector<u64>& in, std::vector<u64>& out, std::string& err);

// Level schedule of an encoded tape for the cooperative value/record sweeps, in which the
// warps of a CTA share one 32-instance tile: the instructions are grouped into levels whose
// members are independent (no member reads a value another member defines, no two members
// write one slot, no member overwrites a slot another member reads), so the warps execute a
// level in any order and synchronise between levels. Slots are renamed for the level order
// (a slot freed by a value's last use is reused from the next level on). Every instruction
// computes the same operation on the same operand values as in `in`, so results are the same
// bits; `pidx` keeps each instruction's recorded-partial index of the order of `in`, so the
// partials land where the derivative sweeps (which walk `in`) read them.
struct Levels {
  std::vector<u64> code;   // instructions level by level (NOPs dropped)
  std::vector<int> begin;  // level l is code[begin[l] .. begin[l+1])
  std::vector<int> pidx;   // per instruction of `code`: its first recorded partial
  std::vector<int> src;    // per instruction of `code`: its index in `in`
  int sz_w = 0;            // work-vector length of the renamed slots
};

// `width`: at most this many instructions per level. Priority: position in `in`; the earliest
// ready instruction always runs, later ones join a level only while fewer than `slot_cap`
// values are live or a slot is free.
// Returns the number of levels, or -1 with `err` set.
// With `ordered_users` the users of every non-constant value also keep their order of `in`
// across levels (no two in one level), as the cooperative reverse sweep needs.
int level_schedule(const std::vector<u64>& in, int width, int slot_cap, Levels& out,
                   std::string& err, bool ordered_users = false);

}  // namespace cgb
