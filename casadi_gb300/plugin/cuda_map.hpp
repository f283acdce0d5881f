// CudaMap: Function::map(n, "cuda") for CasADi, on the GB300 library's C ABI.
//
// A Map (casadi/core/map.hpp:39-327) whose eval, sp_forward and sp_reverse run over all n
// instances at once on the GPU instead of instance by instance (Map::eval_gen,
// casadi/core/map.cpp:141-157; OmpMap::eval, :340-386; Map::sp_forward/sp_reverse, :164-184).
// The buffers are the Map's own (the caller owns arg/res/iw/w, instance-major: input j of
// instance i at arg[j] + i*nnz_in(j)); the tape is taken once, in init, from the wrapped SX
// Function through the public instruction accessors (casadi/core/function.hpp:1109-1151), and
// registered with the library on the first evaluation, so building the Function needs no GPU. Each memory object owns one library memory object (its stream and staging buffers). A
// failing library call returns 1 with the library's message as a warning, like the other Map
// kinds' error flag; nothing throws across the C ABI.
//
// Building: compile this file against the CasADi headers and link libcasadi and
// libcasadi_gb300. Map::create's string switch (map.cpp:39-51) gets one branch returning
// CudaMap::create(f, n) for "cuda"; until a CasADi build carries it, CudaMap::create builds
// the Function directly. Map::deserialize's class-name switch (map.cpp:110-122) gets one
// branch returning CudaMap::deserialize(s) for "CudaMap" (Map::serialize_type writes the
// class name), so a serialized cuda map reads back as one.
#pragma once

#include <mutex>
#include <vector>

#include <casadi/core/map.hpp>

#include "../../include/casadi_gb300.h"

namespace casadi {

class CudaMap : public Map {
 public:
  CudaMap(const std::string& name, const Function& f, casadi_int n) : Map(name, f, n) {}
  ~CudaMap() override;

  // the "CudaMap" branch of Map::deserialize: the Map's fields from the stream, then the tape
  // records from the deserialized Function (a deserialized Function is finalized, not
  // initialised again)
  explicit CudaMap(DeserializingStream& s);
  static ProtoFunction* deserialize(DeserializingStream& s) { return new CudaMap(s); }

  // Function::map(n, "cuda") of f
  static Function create(const Function& f, casadi_int n);

  std::string class_name() const override { return "CudaMap"; }
  bool is_a(const std::string& type, bool recursive) const override {
    return type == "CudaMap" || Map::is_a(type, recursive);
  }
  std::string parallelization() const override { return "cuda"; }

  void init(const Dict& opts) override;
  void* alloc_mem() const override;
  int init_mem(void* mem) const override;
  void free_mem(void* mem) const override;

  int eval(const double** arg, double** res, casadi_int* iw, double* w,
           void* mem) const override;
  int sp_forward(const bvec_t** arg, bvec_t** res, casadi_int* iw, bvec_t* w,
                 void* mem) const override;
  int sp_reverse(bvec_t** arg, bvec_t** res, casadi_int* iw, bvec_t* w,
                 void* mem) const override;

  // the library's tape id (-1: not created yet)
  int tape() const { return tape_; }

 private:
  int ensure(void* mem) const;
  void take_tape();
  std::vector<casadi_gb300_atomic> alg_;
  std::vector<int> nnz_in_, nnz_out_;
  int sz_w_ = 0;
  mutable std::mutex tape_mtx_;
  mutable int tape_ = -1;
};

}  // namespace casadi
