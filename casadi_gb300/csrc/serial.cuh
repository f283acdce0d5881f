// Decoder for Functions serialized by CasADi (host code, no libcasadi).
//
// Reads the text CasADi's SerializingStream writes (casadi/core/serializing_stream.cpp): every
// byte as two letters 'a'+low nibble, 'a'+high nibble; a header (check value 123456789012345,
// protocol version 3, debug flag); little-endian primitives; in debug mode a one-byte type tag
// before each primitive and a descriptor string before each named field; shared objects
// (Sparsity, SX nodes, Functions, GenericType values) as 'd' + definition on first use and
// 'r' + index afterwards, indices counted over all shared objects in the order their
// definitions end. Two top-level forms are accepted: Function::serialize() (function.cpp:
// 1477-1489) and Function::save / StringSerializer / FileSerializer (serializer.cpp: a type
// byte, then the Function as a shared object, or a vector of them as casadi_c_push_file reads,
// casadi_c.cpp:73-94).
//
// SXFunction bodies are read completely (sx_function.cpp:1926-1997): the algorithm, work-vector
// size and the call records of nested SXFunctions. For any other Function class at the top
// level the common part (ProtoFunction and FunctionInternal bodies, function_internal.cpp:
// 4175-4390; for an MXFunction also the XFunction version and input count) is read and the
// body stops there.
#pragma once

#include <string>
#include <vector>

#include "../../include/casadi_gb300.h"

namespace cgb {

struct SerialSparsity {
  bool null = true;
  long long nrow = 0, ncol = 0, nnz = 0;
};

// One OP_CALL record of an SXFunction (ExtendedAlgEl, sx_function.hpp:287-304): the called
// function (index into SerialModel::functions) and its input/output work-vector slots.
struct SerialCall {
  int fn = -1;
  std::vector<int> dep, res;
};

struct SerialFunction {
  std::string cls, name;
  int v_proto = 0, v_internal = 0, v_x = 0, v_sx = 0;  // versions of the bodies read
  std::vector<std::string> name_in, name_out;
  std::vector<SerialSparsity> sp_in, sp_out;
  bool complete = false;  // the whole body was read (SXFunction)
  long long x_inputs = -1;  // XFunction::in entries (SX/MXFunction; read before stopping)
  // SXFunction only
  std::vector<casadi_gb300_atomic> alg;
  long long sz_w = 0;
  long long n_free = 0;  // free variables (the reference refuses to evaluate those)
  std::vector<double> default_in;
  std::vector<SerialCall> calls;
};

struct SerialModel {
  std::vector<SerialFunction> functions;  // called functions before their callers
  std::vector<int> tops;  // the serialized Function(s) (-1: a null Function)
  int top = -1;           // tops[0] when exactly one Function was serialized
  bool debug = false;
  bool saved_form = false;  // written by Function::save / a SerializerBase (type byte first)
};

// Decodes `len` characters of serialized text. Returns 0, or CASADI_GB300_ERR_ARG (malformed
// or truncated text, with the byte offset in `err`) / CASADI_GB300_ERR_UNSUPPORTED (a class
// this decoder does not read, nested inside the function).
int decode_serialized(const char* text, size_t len, SerialModel& out, std::string& err);

// JSON summary of a decoded model (class, name, versions, inputs/outputs with their
// sparsity sizes, and for SXFunctions the tape sizes and call count).
std::string describe_serialized(const SerialModel& m);

}  // namespace cgb
