// pdt_ops.h -- operator objects behind pdt_op (OperatorBase<InputType, OutputType>, operatorbase.h:196-507).
#pragma once

#include <map>
#include <memory>
#include <string>
#include <vector>

#include "pdt_internal.h"

namespace pdt {

typedef std::vector<int64_t> Dims;  // ImageUtilities order, fastest first

std::string dims_str(const Dims& d);

// A positional constant (DataItem, operatorbase.h:160-192): device copy plus a host copy for the small
// ones the engine needs to plan with (masks, trajectories).
struct Constant {
  pdt_dtype dtype;
  Dims size;
  DevBuf dev;
  std::vector<unsigned char> host;  // kept for F32 constants
  size_t numel() const;
  size_t elem_bytes() const { return dtype == PDT_C64 ? 8 : 4; }
};

// Hooks the iterative solvers drive. K-space data is held in an operator-specific compact layout
// (for Cartesian operators: only phase-encode columns with a non-zero mask entry).
struct SolverHooks {
  virtual ~SolverHooks() = default;
  virtual size_t compact_elems() = 0;
  // dense user k-space -> compact layout
  virtual void gather(const float2* dense, float2* compact, cudaStream_t st) = 0;
  // compact layout -> dense user k-space (entries the compact layout does not hold are written as 0)
  virtual void scatter(const float2* compact, float2* dense, cudaStream_t st) = 0;
  // One operator round of a primal-dual iteration:
  //   r <- (r + sigma (K ubar - f)) / (1 + sigma lambda);   khr <- K^H r
  // khr receives `groups()` partial sums spaced `group_stride()` elements apart.
  // `tick`, when non-null, is incremented once by the round's first kernel (the solvers' device-side
  // iteration counter).
  // `dual`, when non-null, is a dual update the round runs inside one of its launches, after that
  // launch's programmatic wait (only where can_fuse_dual says so).
  virtual void round(const float2* ubar, float2* r, const float2* fc, float sigma, float lambda, float2* khr,
                     int* tick, cudaStream_t st, PhaseMarker* mk = nullptr, const DualStep* dual = nullptr) = 0;
  // Whether round() can run a W x H dual update in blocks its launches leave idle.
  virtual bool can_fuse_dual(int W, int H) { return false; }
  // While on, the rounds launch beside other problems' kernels (batched solves): prefer kernels that
  // leave room on each SM over the ones fastest alone.
  virtual void set_concurrent(bool on) {}
  virtual int groups() = 0;
  virtual long long group_stride() = 0;
  // img <- K^H f from the compact layout (the solver's initial u0 = A^T f).
  virtual void adjoint_compact(const float2* fc, float2* img, cudaStream_t st) = 0;
};

class OpImpl {
 public:
  OpImpl(pdt_op_kind kind, std::string name, unsigned nreq, std::map<std::string, std::string> cfg)
      : kind_(kind), name_(std::move(name)), nreq_(nreq), cfg_(std::move(cfg)), gen_(next_generation()) {}
  virtual ~OpImpl() = default;

  // Process-wide unique identity of this operator and its current constants: changes whenever a constant
  // is added, so solvers re-gather their data and re-capture graphs that baked in the operator's tables.
  uint64_t generation() const { return gen_; }

  pdt_op_kind kind() const { return kind_; }
  const std::string& name() const { return name_; }
  std::string print() const;

  // OperatorBase::addConstant (operatorbase.h:238-257)
  void add_constant(pdt_dtype dtype, const Dims& size, const void* data, bool is_device);
  // Replaces constant idx (same type and rank), stream-ordered on st (no counterpart in the reference).
  void replace_constant(unsigned idx, pdt_dtype dtype, const Dims& size, const void* data, bool is_device,
                        cudaStream_t st);

  // OperatorBase::forward / adjoint with operatorCheck (operatorbase.h:297-312, 491-506); device pointers.
  void forward(const float2* src, const Dims& src_size, float2* dst, const Dims& dst_size, cudaStream_t st);
  void adjoint(const float2* src, const Dims& src_size, float2* dst, const Dims& dst_size, cudaStream_t st);

  virtual Dims input_size(const Dims& out) = 0;
  // The image size the constants imply (used by the adjointness check).
  virtual Dims natural_input_size() = 0;
  virtual Dims output_size(const Dims& in) = 0;
  virtual SolverHooks* hooks() = 0;

  // Launch configuration chosen by the operator's autotuner ("" when it has none).
  virtual std::string tuning() { return ""; }

  // Raises (and clears) what the operator's kernels reported on the device since the last check: a
  // bounded wait that gave up (PDT_ERR_TIMEOUT). Reads device memory: call only where the caller waits
  // for the work anyway.
  virtual void check_device_errors() {}

  // Checks for solvers: constants complete, sizes consistent.
  void operator_check(const Dims& in, const Dims& out);

 protected:
  virtual void size_check(const Dims& in, const Dims& out) = 0;
  virtual void execute_forward(const float2* src, float2* dst, cudaStream_t st) = 0;
  virtual void execute_adjoint(const float2* src, float2* dst, cudaStream_t st) = 0;
  // Constant `idx` with the expected type and rank (OperatorBase::getConstant, operatorbase.h:262-290).
  Constant& constant(unsigned idx, pdt_dtype dtype, int ndim);
  // Called when constants change.
  virtual void invalidate() {}

  pdt_op_kind kind_;
  std::string name_;
  unsigned nreq_;
  std::map<std::string, std::string> cfg_;
  std::vector<std::unique_ptr<Constant>> constants_;
  uint64_t gen_;

  static uint64_t next_generation();
};

std::shared_ptr<OpImpl> make_operator(pdt_op_kind kind, const std::map<std::string, std::string>& cfg);

// IU_SIZE_CHECK equivalent.
void size_check_eq(const Dims& a, const Dims& b);

}  // namespace pdt
