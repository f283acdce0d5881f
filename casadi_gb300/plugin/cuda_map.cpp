// CudaMap: see cuda_map.hpp.
#include "cuda_map.hpp"

#include <cstdint>
#include <vector>

#include <casadi/core/calculus.hpp>

namespace casadi {

namespace {

// Memory object: the Function's bookkeeping plus one library memory object.
struct CudaMapMemory : public ProtoFunctionMemory {
  int lib_mem = -1;
};

int lib_mem_of(void* mem) { return static_cast<CudaMapMemory*>(mem)->lib_mem; }

int status(int st) {
  if (st == 0) return 0;
  casadi_warning(std::string("CudaMap: ") + casadi_gb300_last_error());
  return 1;
}

}  // namespace

CudaMap::~CudaMap() {
  clear_mem();
  if (tape_ >= 0) casadi_gb300_tape_free(tape_);
}

Function CudaMap::create(const Function& f, casadi_int n) {
  std::string suffix = str(n) + "_" + f.name();
  return Function::create(new CudaMap("cudamap" + suffix, f, n), Dict());
}

void CudaMap::init(const Dict& opts) {
  Map::init(opts);
  take_tape();
}

CudaMap::CudaMap(DeserializingStream& s) : Map(s) { take_tape(); }

void CudaMap::take_tape() {
  casadi_assert(f_.is_a("SXFunction"), "CudaMap needs an SX Function, got " + f_.class_name());
  // the algorithm through the public accessors, in the ScalarAtomic layout the library takes
  const casadi_int n_instr = f_.n_instructions();
  alg_.assign(n_instr, casadi_gb300_atomic());
  for (casadi_int k = 0; k < n_instr; ++k) {
    casadi_gb300_atomic& e = alg_[k];
    e.op = static_cast<int>(f_.instruction_id(k));
    const std::vector<casadi_int> o = f_.instruction_output(k);
    const std::vector<casadi_int> i = f_.instruction_input(k);
    if (e.op == OP_CONST) {
      e.i0 = static_cast<int>(o.at(0));
      e.a.d = f_.instruction_constant(k);
    } else if (e.op == OP_OUTPUT) {  // i0 output index, i1 slot, i2 nonzero
      e.i0 = static_cast<int>(o.at(0));
      e.a.i[0] = static_cast<int>(i.at(0));
      e.a.i[1] = static_cast<int>(o.at(1));
    } else if (e.op == OP_INPUT) {   // i0 slot, i1 input index, i2 nonzero
      e.i0 = static_cast<int>(o.at(0));
      e.a.i[0] = static_cast<int>(i.at(0));
      e.a.i[1] = static_cast<int>(i.at(1));
    } else {
      e.i0 = static_cast<int>(o.at(0));
      e.a.i[0] = i.empty() ? 0 : static_cast<int>(i[0]);
      e.a.i[1] = i.size() > 1 ? static_cast<int>(i[1]) : e.a.i[0];
    }
  }
  nnz_in_.resize(n_in_);
  nnz_out_.resize(n_out_);
  for (casadi_int j = 0; j < n_in_; ++j) nnz_in_[j] = static_cast<int>(f_.nnz_in(j));
  for (casadi_int j = 0; j < n_out_; ++j) nnz_out_[j] = static_cast<int>(f_.nnz_out(j));
  sz_w_ = static_cast<int>(f_.sz_w());
}

void* CudaMap::alloc_mem() const { return new CudaMapMemory(); }

int CudaMap::init_mem(void* mem) const { return Map::init_mem(mem); }

// The device side, made on first use (construction checks out a memory object too, and must
// not need a GPU): the tape, once per Function, and the memory object's library memory.
int CudaMap::ensure(void* mem) const {
  {
    std::lock_guard<std::mutex> lk(tape_mtx_);
    if (tape_ < 0) {
      const int id = casadi_gb300_tape_create(alg_.data(), static_cast<int>(alg_.size()),
                                              static_cast<int>(n_in_), nnz_in_.data(),
                                              static_cast<int>(n_out_), nnz_out_.data(), sz_w_);
      if (id < 0) return status(id);
      tape_ = id;
    }
  }
  CudaMapMemory* m = static_cast<CudaMapMemory*>(mem);
  if (m->lib_mem < 0) {
    const int id = casadi_gb300_checkout();
    if (id < 0) return status(id);
    m->lib_mem = id;
  }
  return 0;
}

void CudaMap::free_mem(void* mem) const {
  CudaMapMemory* m = static_cast<CudaMapMemory*>(mem);
  if (m->lib_mem >= 0) casadi_gb300_release(m->lib_mem);
  delete m;
}

int CudaMap::eval(const double** arg, double** res, casadi_int* iw, double* w,
                  void* mem) const {
  setup(mem, arg, res, iw, w);
  if (ensure(mem)) return 1;
  return status(casadi_gb300_map_eval(tape_, lib_mem_of(mem), n_, arg, res));
}

int CudaMap::sp_forward(const bvec_t** arg, bvec_t** res, casadi_int* iw, bvec_t* w,
                        void* mem) const {
  static_assert(sizeof(bvec_t) == sizeof(uint64_t), "bvec_t is 64 bits");
  if (ensure(mem)) return 1;
  return status(casadi_gb300_map_sp_forward(tape_, lib_mem_of(mem), n_,
                                            reinterpret_cast<const uint64_t* const*>(arg),
                                            reinterpret_cast<uint64_t* const*>(res)));
}

int CudaMap::sp_reverse(bvec_t** arg, bvec_t** res, casadi_int* iw, bvec_t* w,
                        void* mem) const {
  if (ensure(mem)) return 1;
  return status(casadi_gb300_map_sp_reverse(tape_, lib_mem_of(mem), n_,
                                            reinterpret_cast<uint64_t* const*>(arg),
                                            reinterpret_cast<uint64_t* const*>(res)));
}

}  // namespace casadi
