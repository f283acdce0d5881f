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

}  // namespace cgb
