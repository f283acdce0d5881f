// Decoder for Functions serialized by CasADi: see serial.cuh. Host code only.
//
// The reader follows the deserializing constructors of the reference field by field, with
// their version branches:
//   stream primitives, shared objects  casadi/core/serializing_stream.cpp:45-118, :140-330,
//                                      serializing_stream.hpp:115-205
//   Function, null flag                function.cpp:1482-1496; serializer.cpp:134-138
//   ProtoFunction body (versions 1-2)  function_internal.cpp:4175-4183
//   FunctionInternal body (1-8)        function_internal.cpp:4269-4391
//   XFunction body (1)                 x_function.hpp:307-320
//   SXFunction body (1-3)              sx_function.cpp:1926-1997
//   SX nodes                           sx_node.cpp:238-274, constant_sx.hpp:506-529,
//                                      symbolic_sx.hpp:73-81, unary_sx.hpp:123-131,
//                                      binary_sx.hpp:135-150, call_sx.hpp:156-166,
//                                      output_sx.hpp:147-158
//   Sparsity                           sparsity.cpp:2079-2095 (compressed column format)
//   GenericType                        generic_type.cpp:773-817, generic_type_internal.hpp
#include "serial.cuh"

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <sstream>

namespace cgb {
namespace {

// CasADi operation ids (casadi/core/calculus.hpp:60-218) the node reader dispatches on
constexpr long long kOpConst = 44, kOpParameter = 47, kOpCall = 48, kOpOutputNode = -1;

// casadi_math::is_binary / is_unary (calculus.hpp:1507-1559, :1612-1630)
bool op_binary(long long op) {
  switch (op) {
    case 1: case 2: case 3: case 4: case 8: case 9: case 19: case 20: case 21: case 22:
    case 24: case 25: case 31: case 28: case 97: case 34: case 35: case 43: case 87: case 88:
    case 95: case 32:
      return true;
    default:
      return false;
  }
}

bool op_unary(long long op) {
  switch (op) {
    case 0: case 5: case 6: case 7: case 10: case 11: case 12: case 13: case 14: case 15:
    case 16: case 17: case 18: case 26: case 27: case 23: case 33: case 29: case 30: case 36:
    case 37: case 38: case 39: case 40: case 41: case 42: case 86: case 93: case 94:
      return true;
    default:
      return false;
  }
}

// GenericType ids (generic_type.hpp:43-63)
enum {
  OT_NULL, OT_BOOL, OT_INT, OT_DOUBLE, OT_STRING, OT_INTVECTOR, OT_INTVECTORVECTOR,
  OT_BOOLVECTOR, OT_DOUBLEVECTOR, OT_DOUBLEVECTORVECTOR, OT_STRINGVECTOR, OT_DICT, OT_FUNCTION,
  OT_FUNCTIONVECTOR, OT_VOIDPTR, OT_UNKNOWN, OT_STRINGVECTORVECTOR, OT_DICTVECTOR,
  OT_VECTORVECTOR, OT_VECTOR
};

constexpr long long kCheck = 123456789012345LL;
constexpr long long kProtocol = 3;
// SerializerBase::SERIALIZED_FUNCTION / _FUNCTION_VECTOR (serializer.hpp:78-102)
constexpr int kSerializedFunction = 5, kSerializedFunctionVector = 15;

struct DecodeError {
  int code;
  std::string msg;
};

class Reader {
 public:
  Reader(std::vector<unsigned char> bytes, SerialModel& m) : b_(std::move(bytes)), m_(m) {}

  void run() {
    // header: always without debug decorations (the flag is read last)
    if (raw_i64() != kCheck) fail("not a CasADi serialization (sanity check value differs)");
    const long long v = raw_i64();
    if (v != kProtocol)
      fail("serialization protocol " + std::to_string(v) + ", only 3 is read");
    debug_ = byte() != 0;
    m_.debug = debug_;
    if (pos_ >= b_.size()) fail("no object after the header");
    if (b_[pos_] == kSerializedFunction) {
      // Function::save / SerializerBase::pack(Function): type byte, then a shared Function
      ++pos_;
      m_.saved_form = true;
      partial_ok_ = true;
      m_.tops.push_back(function(nullptr));
    } else if (b_[pos_] == kSerializedFunctionVector) {
      // SerializerBase::pack(std::vector<Function>): type byte, then the vector; a Function
      // whose body is not read can only be the last one
      ++pos_;
      m_.saved_form = true;
      const long long n = count(nullptr, 'V');
      for (long long k = 0; k < n; ++k) {
        partial_ok_ = k == n - 1;
        m_.tops.push_back(function(nullptr));
      }
    } else {
      // Function::serialize(): the Function body directly
      partial_ok_ = true;
      m_.tops.push_back(function_body());
    }
    if (m_.tops.size() == 1) m_.top = m_.tops[0];
  }

 private:
  std::vector<unsigned char> b_;
  size_t pos_ = 0;
  bool debug_ = false;
  SerialModel& m_;
  // shared objects in definition order: kind ('S' sparsity, 'E' SX node, 'F' Function,
  // 'G' GenericType) and, for sparsities and Functions, the index of the decoded value
  struct Shared {
    char kind;
    int idx;
  };
  std::vector<Shared> shared_;
  std::vector<SerialSparsity> sparsities_;

  [[noreturn]] void fail(const std::string& what, int code = CASADI_GB300_ERR_ARG) {
    throw DecodeError{code, what + " (at byte " + std::to_string(pos_) + ")"};
  }

  unsigned char byte() {
    if (pos_ >= b_.size()) fail("truncated serialization");
    return b_[pos_++];
  }
  long long raw_i64() {
    unsigned long long v = 0;
    for (int j = 0; j < 8; ++j) v |= static_cast<unsigned long long>(byte()) << (8 * j);
    return static_cast<long long>(v);
  }
  int raw_i32() {
    unsigned v = 0;
    for (int j = 0; j < 4; ++j) v |= static_cast<unsigned>(byte()) << (8 * j);
    return static_cast<int>(v);
  }

  // debug mode: the one-byte type tag of a primitive, and the descriptor of a named field
  void deco(char c) {
    if (!debug_) return;
    const unsigned char t = byte();
    if (t != static_cast<unsigned char>(c))
      fail(std::string("type tag '") + static_cast<char>(t) + "' where '" + c + "' was written");
  }
  void descr(const char* d) {
    if (!debug_ || d == nullptr) return;
    const std::string got = str_plain();
    if (got != d) fail("field '" + got + "' where '" + d + "' was expected");
  }

  std::string str_plain() {
    deco('s');
    deco('i');
    const int n = raw_i32();
    if (n < 0 || static_cast<size_t>(n) > b_.size() - pos_) fail("bad string length");
    std::string s(reinterpret_cast<const char*>(b_.data() + pos_), static_cast<size_t>(n));
    pos_ += static_cast<size_t>(n);
    return s;
  }

  // named primitives (casadi_int 'J', size_t 'K', int 'i', bool 'b', double 'd', char none)
  long long i64(const char* d) {
    descr(d);
    deco('J');
    return raw_i64();
  }
  long long size(const char* d) {
    descr(d);
    deco('K');
    return raw_i64();
  }
  int i32(const char* d) {
    descr(d);
    deco('i');
    return raw_i32();
  }
  bool boolean(const char* d) {
    descr(d);
    deco('b');
    return byte() != 0;
  }
  double dbl(const char* d) {
    descr(d);
    deco('d');
    unsigned long long v = static_cast<unsigned long long>(raw_i64());
    double x;
    std::memcpy(&x, &v, 8);
    return x;
  }
  char ch(const char* d) {
    descr(d);
    return static_cast<char>(byte());
  }
  std::string str(const char* d) {
    descr(d);
    return str_plain();
  }
  long long count(const char* d, char tag) {
    descr(d);
    deco(tag);
    const long long n = i64(nullptr);
    if (n < 0 || static_cast<unsigned long long>(n) > b_.size()) fail("bad element count");
    return n;
  }
  int version(const char* name, int lo, int hi) {
    const int v = i32((std::string(name) + "::serialization::version").c_str());
    if (v < lo || v > hi)
      fail(std::string(name) + " body of version " + std::to_string(v) + ", readable: " +
           std::to_string(lo) + ".." + std::to_string(hi));
    return v;
  }

  // vectors of primitives
  std::vector<bool> bools(const char* d) {
    std::vector<bool> v(static_cast<size_t>(count(d, 'V')));
    for (size_t k = 0; k < v.size(); ++k) v[k] = boolean(nullptr);
    return v;
  }
  std::vector<std::string> strings(const char* d) {
    std::vector<std::string> v(static_cast<size_t>(count(d, 'V')));
    for (auto& s : v) s = str(nullptr);
    return v;
  }
  std::vector<long long> ints64(const char* d) {
    std::vector<long long> v(static_cast<size_t>(count(d, 'V')));
    for (auto& x : v) x = i64(nullptr);
    return v;
  }
  std::vector<int> ints32(const char* d) {
    std::vector<int> v(static_cast<size_t>(count(d, 'V')));
    for (auto& x : v) x = i32(nullptr);
    return v;
  }
  std::vector<double> doubles(const char* d) {
    std::vector<double> v(static_cast<size_t>(count(d, 'V')));
    for (auto& x : v) x = dbl(nullptr);
    return v;
  }

  // shared objects: 'd' + definition, or 'r' + index of an earlier definition
  char shared_flag() {
    const char f = ch("Shared::flag");
    if (f != 'd' && f != 'r') fail(std::string("bad shared-object flag '") + f + "'");
    return f;
  }
  const Shared& reference(char kind) {
    const long long k = i64("Shared::reference");
    if (k < 0 || static_cast<size_t>(k) >= shared_.size()) fail("shared reference out of range");
    const Shared& s = shared_[static_cast<size_t>(k)];
    if (s.kind != kind) fail(std::string("shared reference to a '") + s.kind + "' object");
    return s;
  }

  int sparsity(const char* d) {
    descr(d);
    deco('S');
    if (shared_flag() == 'r') return reference('S').idx;
    // compressed (sparsity.cpp:1321-1372): nrow, ncol, colind[ncol+1], row[nnz], or the dense
    // shorthand nrow, ncol, 1 (a canonical colind starts at 0); empty: the null sparsity
    const std::vector<long long> c = ints64("SparsityInternal::compressed");
    SerialSparsity sp;
    if (!c.empty()) {
      if (c.size() < 3) fail("short compressed sparsity");
      const long long nr = c[0], nc = c[1];
      if (nr < 0 || nc < 0) fail("negative sparsity dimensions");
      sp.null = false;
      sp.nrow = nr;
      sp.ncol = nc;
      if (c[2] == 1) {
        if (c.size() != 3) fail("dense sparsity shorthand of inconsistent length");
        sp.nnz = nr * nc;
      } else {
        if (static_cast<long long>(c.size()) < 3 + nc) fail("short compressed sparsity");
        sp.nnz = c[static_cast<size_t>(2 + nc)];
        if (sp.nnz < 0 || static_cast<long long>(c.size()) != 3 + nc + sp.nnz)
          fail("compressed sparsity of inconsistent length");
      }
    }
    sparsities_.push_back(sp);
    const int idx = static_cast<int>(sparsities_.size()) - 1;
    shared_.push_back({'S', idx});
    return idx;
  }

  // one SX node (definition or reference), read with an explicit stack so deep expression
  // graphs do not recurse; unary/binary/output/call nodes are complete once their
  // dependencies are read, and a node's shared index is taken when it is complete
  void sx_elem(const char* d) {
    struct Frame {
      long long op, need, got;
    };
    std::vector<Frame> st;
    const char* dd = d;
    for (;;) {
      descr(dd);
      deco('E');
      bool value_ready = false;
      if (shared_flag() == 'r') {
        reference('E');
        value_ready = true;
      } else {
        const long long op = i64("SXNode::op");
        if (op_binary(op)) {
          st.push_back({op, 2, 0});
          dd = "UnarySX::dep0";
        } else if (op_unary(op)) {
          st.push_back({op, 1, 0});
          dd = "UnarySX::dep";
        } else if (op == kOpParameter) {
          str("SymbolicSX::name");
          shared_.push_back({'E', 0});
          value_ready = true;
        } else if (op == kOpConst) {
          const char t = ch("ConstantSX::type");
          if (t == 'r') {
            dbl("ConstantSX::value");
          } else if (t == 'i') {
            i32("ConstantSX::value");
          } else if (!std::strchr("01nfFm", t) || t == 0) {
            fail(std::string("unknown constant kind '") + t + "'");
          }
          shared_.push_back({'E', 0});
          value_ready = true;
        } else if (op == kOpOutputNode) {
          st.push_back({op, 1, 0});
          dd = "OutputSX::dep";
        } else if (op == kOpCall) {
          function("CallSX::f");
          const long long n = count("CallSX::dep", 'V');
          if (n == 0) {
            shared_.push_back({'E', 0});
            value_ready = true;
          } else {
            st.push_back({op, n, 0});
            dd = nullptr;
          }
        } else {
          fail("SX node with operation " + std::to_string(op), CASADI_GB300_ERR_UNSUPPORTED);
        }
      }
      if (!value_ready) continue;
      // deliver the finished node to the frames waiting for it
      for (;;) {
        if (st.empty()) return;
        Frame& f = st.back();
        if (++f.got < f.need) {
          dd = f.op == kOpCall ? nullptr : "UnarySX::dep1";
          break;
        }
        if (f.op == kOpOutputNode) i32("OutputSX::oind");
        st.pop_back();
        shared_.push_back({'E', 0});
      }
    }
  }

  void sx_elems(const char* d) {
    const long long n = count(d, 'V');
    for (long long k = 0; k < n; ++k) sx_elem(nullptr);
  }

  // Matrix<SXElem> (matrix_impl.hpp:3049-3061): sparsity, then the nonzeros
  void sx_matrix() {
    sparsity("Matrix::sparsity");
    sx_elems("Matrix::nonzeros");
  }
  void sx_matrices(const char* d) {
    const long long n = count(d, 'V');
    for (long long k = 0; k < n; ++k) sx_matrix();
  }

  // Functions and GenericType values nest by recursion; a depth limit keeps corrupted or
  // hostile text from exhausting the stack
  static constexpr int kMaxDepth = 200;
  int depth_ = 0;
  struct Nest {
    Reader& r;
    explicit Nest(Reader& rr) : r(rr) {
      if (++r.depth_ > kMaxDepth) r.fail("objects nested deeper than " + std::to_string(kMaxDepth));
    }
    ~Nest() { --r.depth_; }
  };

  void generic(const char* d) {
    descr(d);
    deco('G');
    if (shared_flag() == 'r') {
      reference('G');
      return;
    }
    Nest nest(*this);
    const int type = i32("GenericType::type");
    const char* v = "GenericType::d";
    switch (type) {
      case OT_BOOL: boolean(v); break;
      case OT_INT: i64(v); break;
      case OT_DOUBLE: dbl(v); break;
      case OT_STRING: str(v); break;
      case OT_INTVECTOR: ints64(v); break;
      case OT_INTVECTORVECTOR: {
        const long long n = count(v, 'V');
        for (long long k = 0; k < n; ++k) ints64(nullptr);
      } break;
      case OT_DOUBLEVECTOR: doubles(v); break;
      case OT_DOUBLEVECTORVECTOR: {
        const long long n = count(v, 'V');
        for (long long k = 0; k < n; ++k) doubles(nullptr);
      } break;
      case OT_STRINGVECTOR: strings(v); break;
      case OT_STRINGVECTORVECTOR: {
        const long long n = count(v, 'V');
        for (long long k = 0; k < n; ++k) strings(nullptr);
      } break;
      case OT_FUNCTION: function(v); break;
      case OT_FUNCTIONVECTOR: {
        const long long n = count(v, 'V');
        for (long long k = 0; k < n; ++k) function(nullptr);
      } break;
      case OT_DICT: dict(v); break;
      case OT_DICTVECTOR: {
        const long long n = count(v, 'V');
        for (long long k = 0; k < n; ++k) dict(nullptr);
      } break;
      case OT_VECTOR: {
        const long long n = count(v, 'V');
        for (long long k = 0; k < n; ++k) generic(nullptr);
      } break;
      case OT_VECTORVECTOR: {
        const long long n = count(v, 'V');
        for (long long k = 0; k < n; ++k) {
          const long long m = count(nullptr, 'V');
          for (long long j = 0; j < m; ++j) generic(nullptr);
        }
      } break;
      default:
        fail("GenericType of type " + std::to_string(type), CASADI_GB300_ERR_UNSUPPORTED);
    }
    shared_.push_back({'G', 0});
  }

  void dict(const char* d) {
    const long long n = count(d, 'D');
    for (long long k = 0; k < n; ++k) {
      str(nullptr);
      generic(nullptr);
    }
  }

  // a Function as a shared object; returns its index in m_.functions (-1: null)
  int function(const char* d) {
    descr(d);
    deco('F');
    if (shared_flag() == 'r') return reference('F').idx;
    const int idx = function_body();
    shared_.push_back({'F', idx});
    return idx;
  }

  // Function::deserialize: null flag, base class name, body
  int function_body() {
    const bool partial_ok = partial_ok_;
    partial_ok_ = false;  // nested Functions are always read completely
    if (boolean("Function::null")) return -1;
    Nest nest(*this);
    SerialFunction f;
    f.cls = str("FunctionInternal::base_function");
    const bool sx = f.cls == "SXFunction";
    if (!sx && !partial_ok)
      fail(f.cls + " inside the stream (only SXFunctions are read through)",
           CASADI_GB300_ERR_UNSUPPORTED);
    proto_and_internal(f);
    if (sx) {
      sx_body(f);
    } else if (f.cls == "MXFunction") {
      // the MX expressions are not read; the XFunction header still is
      f.v_x = version("XFunction", 1, 1);
      f.x_inputs = count("XFunction::in", 'V');
    }
    m_.functions.push_back(std::move(f));
    return static_cast<int>(m_.functions.size()) - 1;
  }
  bool partial_ok_ = false;  // the next Function read may stop after its common part

  void proto_and_internal(SerialFunction& f) {
    // ProtoFunction (function_internal.cpp:4175-4183)
    f.v_proto = version("ProtoFunction", 1, 2);
    f.name = str("ProtoFunction::name");
    boolean("ProtoFunction::verbose");
    boolean("ProtoFunction::print_time");
    boolean("ProtoFunction::record_time");
    if (f.v_proto >= 2) {
      boolean("ProtoFunction::regularity_check");
      boolean("ProtoFunction::error_on_fail");
    }
    // FunctionInternal (function_internal.cpp:4269-4391)
    const int v = f.v_internal = version("FunctionInternal", 1, 8);
    bools("FunctionInternal::is_diff_in");
    bools("FunctionInternal::is_diff_out");
    for (long long n = count("FunctionInternal::sp_in", 'V'), k = 0; k < n; ++k)
      f.sp_in.push_back(sparsities_[static_cast<size_t>(sparsity(nullptr))]);
    for (long long n = count("FunctionInternal::sp_out", 'V'), k = 0; k < n; ++k)
      f.sp_out.push_back(sparsities_[static_cast<size_t>(sparsity(nullptr))]);
    f.name_in = strings("FunctionInternal::name_in");
    f.name_out = strings("FunctionInternal::name_out");
    boolean("FunctionInternal::jit");
    boolean("FunctionInternal::jit_cleanup");
    const std::string jit_serialize = v >= 2 ? str("FunctionInternal::jit_serialize") : "source";
    if (jit_serialize == "link" || jit_serialize == "embed") {
      str("FunctionInternal::jit_library");
      if (jit_serialize == "embed") {
        // unpack(std::ostream&): 'B', size_t length, the bytes
        descr("FunctionInternal::jit_binary");
        deco('B');
        const long long n = size(nullptr);
        if (n < 0 || static_cast<unsigned long long>(n) > b_.size() - pos_) fail("bad blob size");
        pos_ += static_cast<size_t>(n);
      }
    }
    boolean("FunctionInternal::jit_temp_suffix");
    str("FunctionInternal::jit_base_name");
    dict("FunctionInternal::jit_options");
    str("FunctionInternal::compiler_plugin");
    boolean("FunctionInternal::has_refcount");
    if (v >= 6) dict("FunctionInternal::cache_init");
    function("FunctionInternal::derivative_of");
    dbl("FunctionInternal::jac_penalty");
    for (const char* e :
         {"FunctionInternal::enable_forward", "FunctionInternal::enable_reverse",
          "FunctionInternal::enable_jacobian", "FunctionInternal::enable_fd",
          "FunctionInternal::enable_forward_op", "FunctionInternal::enable_reverse_op",
          "FunctionInternal::enable_jacobian_op", "FunctionInternal::enable_fd_op"})
      boolean(e);
    dbl("FunctionInternal::ad_weight");
    dbl("FunctionInternal::ad_weight_sp");
    boolean("FunctionInternal::always_inline");
    boolean("FunctionInternal::never_inline");
    i64("FunctionInternal::max_num_dir");
    if (v < 3) boolean("FunctionInternal::regularity_check");
    boolean("FunctionInternal::inputs_check");
    dbl("FunctionInternal::fd_step");
    str("FunctionInternal::fd_method");
    boolean("FunctionInternal::print_in");
    boolean("FunctionInternal::print_out");
    if (v >= 7) boolean("FunctionInternal::print_canonical");
    if (v >= 4) i64("FunctionInternal::max_io");
    boolean("FunctionInternal::dump_in");
    boolean("FunctionInternal::dump_out");
    str("FunctionInternal::dump_dir");
    str("FunctionInternal::dump_format");
    dict("FunctionInternal::forward_options");
    dict("FunctionInternal::reverse_options");
    if (v >= 5) {
      dict("FunctionInternal::jacobian_options");
      dict("FunctionInternal::der_options");
    }
    function("FunctionInternal::custom_jacobian");
    if (v >= 8)
      for (long long n = count("FunctionInternal::registered_functions", 'V'), k = 0; k < n; ++k)
        function(nullptr);
    for (const char* e : {"FunctionInternal::sz_arg_per", "FunctionInternal::sz_res_per",
                          "FunctionInternal::sz_iw_per", "FunctionInternal::sz_w_per",
                          "FunctionInternal::sz_arg_tmp", "FunctionInternal::sz_res_tmp",
                          "FunctionInternal::sz_iw_tmp", "FunctionInternal::sz_w_tmp"})
      size(e);
  }

  void sx_body(SerialFunction& f) {
    // XFunction (x_function.hpp:307-312): the symbolic inputs
    f.v_x = version("XFunction", 1, 1);
    f.x_inputs = count("XFunction::in", 'V');
    for (long long k = 0; k < f.x_inputs; ++k) sx_matrix();
    // SXFunction (sx_function.cpp:1926-1997)
    const int v = f.v_sx = version("SXFunction", 1, 3);
    const long long n_instr = size("SXFunction::n_instr");
    // every instruction takes at least 16 bytes further on: bounds the allocation below
    if (n_instr < 0 || static_cast<unsigned long long>(n_instr) > (b_.size() - pos_) / 16)
      fail("bad instruction count");
    f.sz_w = size("SXFunction::worksize");
    const long long n_free = count("SXFunction::free_vars", 'V');
    for (long long k = 0; k < n_free; ++k) sx_elem(nullptr);
    f.n_free = n_free;
    sx_elems("SXFunction::operations");
    sx_elems("SXFunction::constants");
    f.default_in = doubles("SXFunction::default_in");
    if (v >= 2) {
      size("SXFunction::call_sz_arg");
      size("SXFunction::call_sz_res");
      size("SXFunction::call_sz_iw");
      size("SXFunction::call_sz_w");
      size("SXFunction::call_sz_arg");  // sz_w_arg, written under this descriptor
      size("SXFunction::call_sz_res");  // sz_w_res, likewise
      const long long n_el = size("SXFunction::call_el_size");
      if (n_el < 0 || static_cast<unsigned long long>(n_el) > b_.size()) fail("bad call count");
      for (long long k = 0; k < n_el; ++k) {
        SerialCall c;
        c.fn = function("SXFunction::call_el_f");
        if (c.fn < 0) fail("call record of a null Function");
        c.dep = ints32("SXFunction::call_el_dep");
        c.res = ints32("SXFunction::call_el_res");
        ints32("SXFunction::call_el_copy_elision_arg");
        ints32("SXFunction::call_el_copy_elision_offset");
        f.calls.push_back(std::move(c));
      }
      bools("SXFunction::copy_elision");
    }
    f.alg.resize(static_cast<size_t>(n_instr));
    for (auto& e : f.alg) {
      e.op = i32("SXFunction::ScalarAtomic::op");
      e.i0 = i32("SXFunction::ScalarAtomic::i0");
      // i1/i2 share their bytes with the constant of OP_CONST (the ScalarAtomic union)
      e.a.i[0] = i32("SXFunction::ScalarAtomic::i1");
      e.a.i[1] = i32("SXFunction::ScalarAtomic::i2");
    }
    boolean("SXFunction::live_variables");
    if (v >= 3) boolean("SXFunction::print_instructions");
    // the output expressions, written after the algorithm (x_function.hpp:314-320)
    sx_matrices("XFunction::out");
    f.complete = true;
  }
};

void json_str(std::ostringstream& o, const std::string& s) {
  o << '"';
  for (unsigned char c : s) {
    if (c == '"' || c == '\\') {
      o << '\\' << c;
    } else if (c < 0x20) {
      char buf[8];
      std::snprintf(buf, sizeof(buf), "\\u%04x", c);
      o << buf;
    } else {
      o << c;
    }
  }
  o << '"';
}

}  // namespace

int decode_serialized(const char* text, size_t len, SerialModel& out, std::string& err) {
  out = SerialModel();
  if (text == nullptr) {
    err = "null text";
    return CASADI_GB300_ERR_ARG;
  }
  while (len > 0 && (text[len - 1] == '\n' || text[len - 1] == '\r' || text[len - 1] == ' ' ||
                     text[len - 1] == '\t' || text[len - 1] == '\0'))
    --len;
  if (len % 2) {
    err = "serialized text of odd length";
    return CASADI_GB300_ERR_ARG;
  }
  std::vector<unsigned char> bytes(len / 2);
  for (size_t k = 0; k < bytes.size(); ++k) {
    const int lo = static_cast<unsigned char>(text[2 * k]) - 'a';
    const int hi = static_cast<unsigned char>(text[2 * k + 1]) - 'a';
    if (lo < 0 || lo > 15 || hi < 0 || hi > 15) {
      err = "character outside 'a'..'p' at offset " + std::to_string(2 * k);
      return CASADI_GB300_ERR_ARG;
    }
    bytes[k] = static_cast<unsigned char>(lo | (hi << 4));
  }
  try {
    Reader r(std::move(bytes), out);
    r.run();
  } catch (const DecodeError& e) {
    err = e.msg;
    return e.code;
  } catch (const std::exception& e) {
    err = e.what();
    return CASADI_GB300_ERR_ARG;
  }
  return 0;
}

std::string describe_serialized(const SerialModel& m) {
  std::ostringstream o;
  o.precision(17);
  o << "{\"debug\": " << (m.debug ? "true" : "false")
    << ", \"saved_form\": " << (m.saved_form ? "true" : "false") << ", \"functions\": [";
  for (size_t k = 0; k < m.functions.size(); ++k) {
    const SerialFunction& f = m.functions[k];
    if (k) o << ", ";
    o << "{\"class\": ";
    json_str(o, f.cls);
    o << ", \"name\": ";
    json_str(o, f.name);
    o << ", \"versions\": [" << f.v_proto << ", " << f.v_internal << ", " << f.v_x << ", "
      << f.v_sx << "], \"complete\": " << (f.complete ? "true" : "false")
      << ", \"x_inputs\": " << f.x_inputs;
    for (int io = 0; io < 2; ++io) {
      const auto& names = io ? f.name_out : f.name_in;
      const auto& sps = io ? f.sp_out : f.sp_in;
      o << (io ? ", \"outputs\": [" : ", \"inputs\": [");
      for (size_t j = 0; j < sps.size(); ++j) {
        if (j) o << ", ";
        o << "{\"name\": ";
        json_str(o, j < names.size() ? names[j] : std::string());
        o << ", \"size\": [" << sps[j].nrow << ", " << sps[j].ncol << "], \"nnz\": " << sps[j].nnz
          << "}";
      }
      o << "]";
    }
    if (f.complete) {
      o << ", \"n_instr\": " << f.alg.size() << ", \"sz_w\": " << f.sz_w
        << ", \"n_free\": " << f.n_free << ", \"calls\": [";
      for (size_t c = 0; c < f.calls.size(); ++c) o << (c ? ", " : "") << f.calls[c].fn;
      o << "]";
    }
    o << "}";
  }
  o << "], \"top\": " << m.top << ", \"tops\": [";
  for (size_t k = 0; k < m.tops.size(); ++k) o << (k ? ", " : "") << m.tops[k];
  o << "]}";
  return o.str();
}

}  // namespace cgb
