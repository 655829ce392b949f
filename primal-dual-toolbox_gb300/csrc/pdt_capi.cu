// pdt_capi.cu -- C ABI (include/pdt.h): operator and optimizer handles, the solver loops and error
// mapping. Status codes and thread-local messages replace the reference's IuException.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <iostream>
#include <map>
#include <mutex>
#include <tuple>
#include <memory>
#include <random>
#include <sstream>

#include "pdt_ops.h"
#include "pdt_schedule.h"

namespace pdt {

std::atomic<uint64_t> g_launches{0};

bool pdl_enabled() {
  static const bool on = [] {
    const char* e = std::getenv("PDT_LAUNCH_PDL");
    return !(e && e[0] == '0');
  }();
  return on;
}

std::shared_ptr<OpImpl> make_cartesian_operator(pdt_op_kind kind);

std::string dims_str(const Dims& d) {
  std::ostringstream os;
  os << "(";
  for (size_t i = 0; i < d.size(); ++i) os << (i ? ", " : "") << d[i];
  os << ")";
  return os.str();
}

void size_check_eq(const Dims& a, const Dims& b) {
  if (a != b) throw Error(PDT_ERR_SIZE, "Size mismatch: " + dims_str(a) + " != " + dims_str(b));
}

static size_t numel_of(const Dims& d) {
  size_t n = 1;
  for (auto v : d) n *= (size_t)v;
  return n;
}

size_t Constant::numel() const { return numel_of(size); }

// ------------------------------------------------------------------------------------------------
// OperatorBase behaviour (operatorbase.h:196-507)
// ------------------------------------------------------------------------------------------------
std::string OpImpl::print() const {
  std::ostringstream os;
  os << name_ << ": Added constants: (" << constants_.size() << "/" << nreq_ << ")";
  return os.str();
}

void OpImpl::add_constant(pdt_dtype dtype, const Dims& size, const void* data, bool is_device) {
  if (constants_.size() >= nreq_)  // operatorbase.h:241-256
    throw Error(PDT_ERR_CONSTANTS, "Operator '" + name_ + "': Too many InputTypeConstants. Could not add new constant.'");
  auto c = std::make_unique<Constant>();
  c->dtype = dtype;
  c->size = size;
  const size_t bytes = c->numel() * c->elem_bytes();
  c->dev.ensure(std::max<size_t>(bytes, 1));
  if (bytes) {
    PDT_CUDA_CHECK(cudaMemcpy(c->dev.p, data, bytes, is_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice));
    if (dtype == PDT_F32) {
      c->host.resize(bytes);
      PDT_CUDA_CHECK(cudaMemcpy(c->host.data(), data, bytes, is_device ? cudaMemcpyDeviceToHost : cudaMemcpyHostToHost));
    }
  }
  constants_.push_back(std::move(c));
  gen_ = next_generation();
  invalidate();
}

// Replacing a constant keeps its device buffer when the size is unchanged, so graphs and launch
// parameters that point at it stay valid; the copy is ordered on `st`. F32 constants (masks,
// trajectories, density weights) define the operator's tables: an unchanged value is a no-op, a changed
// one waits for the work already queued on `st` (which may still read the tables), then rebuilds them
// and starts a new generation. Complex constants (coil sensitivities) only change values the kernels
// read, so they need neither.
void OpImpl::replace_constant(unsigned idx, pdt_dtype dtype, const Dims& size, const void* data, bool is_device,
                              cudaStream_t st) {
  if (idx >= constants_.size()) {
    std::ostringstream os;
    os << "Operator '" << name_ << "': Requested index (" << idx
       << ") is not valid. Constants available: " << constants_.size();
    throw Error(PDT_ERR_CONSTANTS, os.str());
  }
  Constant& c = *constants_[idx];
  if (c.dtype != dtype || c.size.size() != size.size())
    throw Error(PDT_ERR_CONSTANTS, "Operator '" + name_ + "': constant " + std::to_string(idx) +
                                       " can only be replaced by one of the same type and rank");
  const size_t bytes = numel_of(size) * c.elem_bytes();
  const bool resized = size != c.size;
  bool changed = resized;
  if (dtype == PDT_F32) {
    std::vector<unsigned char> h(bytes);
    if (bytes) {
      if (is_device) {
        PDT_CUDA_CHECK(cudaMemcpyAsync(h.data(), data, bytes, cudaMemcpyDeviceToHost, st));
        PDT_CUDA_CHECK(cudaStreamSynchronize(st));
      } else {
        std::memcpy(h.data(), data, bytes);
      }
    }
    changed = changed || h != c.host;
    if (!changed) return;
    PDT_CUDA_CHECK(cudaStreamSynchronize(st));
    c.host.swap(h);
  }
  if (resized) {
    c.dev.ensure(std::max<size_t>(bytes, 1));
    c.size = size;
  }
  if (bytes)
    PDT_CUDA_CHECK(cudaMemcpyAsync(c.dev.p, data, bytes, is_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                                   st));
  if (changed) {
    gen_ = next_generation();
    invalidate();
  }
}

uint64_t OpImpl::next_generation() {
  static std::atomic<uint64_t> g_gen{0};
  return ++g_gen;
}

Constant& OpImpl::constant(unsigned idx, pdt_dtype dtype, int ndim) {
  if (idx >= constants_.size()) {  // operatorbase.h:266-274
    std::ostringstream os;
    os << "Operator '" << name_ << "': Requested index (" << idx
       << ") is not valid. Constants available: " << constants_.size();
    throw Error(PDT_ERR_CONSTANTS, os.str());
  }
  Constant& c = *constants_[idx];
  if (c.dtype != dtype || (int)c.size.size() != ndim) {  // operatorbase.h:276-287
    std::ostringstream os;
    os << "Operator '" << name_ << "': Data at idx (" << idx
       << ") cannot be cast to type iu::LinearDeviceMemory<PixelType, Ndim> with PixelType="
       << (dtype == PDT_C64 ? "float2" : "float") << " Ndim=" << ndim;
    throw Error(PDT_ERR_CONSTANTS, os.str());
  }
  return c;
}

void OpImpl::operator_check(const Dims& in, const Dims& out) {
  if (constants_.size() != nreq_) {  // operatorbase.h:493-502
    std::ostringstream os;
    os << "Operator '" << name_ << "': Number of constants (" << constants_.size()
       << ") does not match number of required constants (" << nreq_ << ")";
    throw Error(PDT_ERR_CONSTANTS, os.str());
  }
  size_check(in, out);
}

void OpImpl::forward(const float2* src, const Dims& src_size, float2* dst, const Dims& dst_size, cudaStream_t st) {
  operator_check(src_size, dst_size);
  execute_forward(src, dst, st);
}

void OpImpl::adjoint(const float2* src, const Dims& src_size, float2* dst, const Dims& dst_size, cudaStream_t st) {
  operator_check(dst_size, src_size);
  execute_adjoint(src, dst, st);
}

static std::map<std::string, std::string> to_map(const pdt_kv* cfg, int n) {
  std::map<std::string, std::string> m;
  for (int i = 0; i < n; ++i) {
    if (!cfg[i].key || !cfg[i].value) throw Error(PDT_ERR_INVALID_ARGUMENT, "null config key or value");
    m[cfg[i].key] = cfg[i].value;
  }
  return m;
}

std::shared_ptr<OpImpl> make_radial_operator(pdt_op_kind kind, const std::map<std::string, std::string>& cfg);

std::shared_ptr<OpImpl> make_operator(pdt_op_kind kind, const std::map<std::string, std::string>& cfg) {
  switch (kind) {
    case PDT_OP_CARTESIAN:
    case PDT_OP_CARTESIAN_ROOS:
    case PDT_OP_SAMPLING: {
      if (!cfg.empty()) {  // OperatorBase constructor (operatorbase.h:219-228) with min = max = 0
        const char* nm = kind == PDT_OP_CARTESIAN        ? "MriCartesianOperator"
                         : kind == PDT_OP_CARTESIAN_ROOS ? "MriCartesianRemoveROOSOperator"
                                                         : "MriSamplingOperator";
        std::ostringstream os;
        os << "Operator '" << nm << "': Invalid amount of configuration parameters (min: 0 max: 0) required, got ("
           << cfg.size() << ").";
        throw Error(PDT_ERR_CONFIG, os.str());
      }
      return make_cartesian_operator(kind);
    }
    case PDT_OP_RADIAL:
    case PDT_OP_RADIAL_SINGLECOIL:
      return make_radial_operator(kind, cfg);
  }
  throw Error(PDT_ERR_INVALID_ARGUMENT, "unknown operator kind");
}

// ------------------------------------------------------------------------------------------------
// CUDA-graph replay of a fixed number of iterations.
// ------------------------------------------------------------------------------------------------
struct IterGraph {
  cudaGraphExec_t exec = nullptr;
  uint64_t key = 0;
  int iters = 0;
  uint64_t kernels = 0;
  ~IterGraph() { reset(); }
  void reset() {
    if (exec) cudaGraphExecDestroy(exec);
    exec = nullptr;
    key = 0;
  }
};

// Runs `n` iterations of `body(parity)` (parity alternates 0,1,0,...; `n_per_graph` even) on `st`:
// full chunks replay a captured graph, the remainder is launched directly.
static void run_iterations(IterGraph& g, uint64_t key, int n, int n_per_graph,
                           const std::function<void(int, cudaStream_t)>& body, cudaStream_t st, cudaStream_t cap) {
  const int full = n / n_per_graph;
  if (full > 0) {
    if (!g.exec || g.key != key || g.iters != n_per_graph) {
      g.reset();
      const uint64_t before = g_launches.load();
      PDT_CUDA_CHECK(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
      try {
        for (int i = 0; i < n_per_graph; ++i) body(i & 1, cap);
      } catch (...) {
        cudaGraph_t dummy = nullptr;
        cudaStreamEndCapture(cap, &dummy);
        if (dummy) cudaGraphDestroy(dummy);
        throw;
      }
      cudaGraph_t graph = nullptr;
      PDT_CUDA_CHECK(cudaStreamEndCapture(cap, &graph));
      // capturing counted the kernels once; replays count them again below
      g.kernels = g_launches.load() - before;
      g_launches.fetch_sub(g.kernels);
      cudaError_t e = cudaGraphInstantiate(&g.exec, graph, 0);
      cudaGraphDestroy(graph);
      if (e != cudaSuccess) throw Error(PDT_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
      g.key = key;
      g.iters = n_per_graph;
    }
    for (int i = 0; i < full; ++i) {
      PDT_CUDA_CHECK(cudaGraphLaunch(g.exec, st));
      count_launch(g.kernels);
    }
  }
  for (int i = full * n_per_graph; i < n; ++i) body(i & 1, st);
}

// ------------------------------------------------------------------------------------------------
// Optimizers
// ------------------------------------------------------------------------------------------------
enum Field { F_U, F_UB, F_VX, F_VY, F_VBX, F_VBY, F_PX, F_PY, F_QXX, F_QYY, F_QXY, F_COUNT };
constexpr int F_R = F_COUNT;  // the k-space dual r (with-operator optimizers), dense user layout

class OptImpl {
 public:
  OptImpl(pdt_opt_kind kind, pdt_dtype dtype) : kind_(kind), cplx_(dtype == PDT_C64) {
    params_.alpha0 = 1;
    params_.alpha1 = 1;
    params_.lambda = 1;
    params_.reduction = 1;
    params_.max_iter = 1;
    params_.check = 100;
  }
  ~OptImpl() {
    graph_.reset();
    if (own_) cudaStreamDestroy(own_);
    if (cap_) cudaStreamDestroy(cap_);
    if (aux_) cudaStreamDestroy(aux_);
    if (ev_fork_) cudaEventDestroy(ev_fork_);
    if (ev_join_) cudaEventDestroy(ev_join_);
  }

  bool with_op() const { return kind_ == PDT_OPT_TV_OP || kind_ == PDT_OPT_TGV_OP || kind_ == PDT_OPT_TGV_MRI; }
  bool tgv() const { return kind_ == PDT_OPT_TGV || kind_ == PDT_OPT_TGV_OP || kind_ == PDT_OPT_TGV_MRI; }
  size_t pix() const { return cplx_ ? 8 : 4; }
  // Relative cost of one iteration, for spreading a batch over worker streams: the data's elements (coils x
  // k-space samples with an operator) plus the image's pixels.
  size_t work_estimate() const { return numel_of(fsize_) + (size_t)W_ * H_; }

  pdt_params params_;
  // Step sizes of the with-operator solves when positive (pdt_opt_set_steps); 0: the reference's.
  float step_tau_ = 0.f, step_sigma_ = 0.f;

  void set_operator(std::shared_ptr<OpImpl> op) {
    if (!with_op()) throw Error(PDT_ERR_INVALID_ARGUMENT, "this optimizer takes no operator");
    op_ = std::move(op);
    fc_valid_ = false;
    ++version_;
  }

  // setNoisyData (tgvmrioptimizer.cu:81-91, tvoptimizer.cu:68-74)
  void set_noisy_data(const void* f, const Dims& size, bool is_device, cudaStream_t st) {
    if (!with_op() && size.size() != 2) throw Error(PDT_ERR_SIZE, "noisy data must be 2-D, got " + dims_str(size));
    const size_t bytes = numel_of(size) * pix();
    f_.ensure(std::max<size_t>(bytes, 1));
    copy_in(f_.p, f, bytes, is_device, st);
    fsize_ = size;
    has_f_ = true;
    r_reset_ = true;  // r = 0
    fc_valid_ = false;
    ++version_;
  }

  // setInput0 (tgvmrioptimizer.cu:62-79): u = ubar = input; v, vbar, p, q = 0.
  void set_input0(const void* u0, const Dims& size, bool is_device, cudaStream_t st) {
    if (size.size() != 2) throw Error(PDT_ERR_SIZE, "input must be 2-D, got " + dims_str(size));
    alloc_state(size);
    const size_t plane = plane_bytes();
    PDT_CUDA_CHECK(cudaMemsetAsync(img_.p, 0, img_.bytes, st));
    parity_ = 0;
    copy_in(field(F_U, 0), u0, plane, is_device, st);
    PDT_CUDA_CHECK(cudaMemcpyAsync(field(F_UB, 0), field(F_U, 0), plane, cudaMemcpyDeviceToDevice, st));
    has_state_ = true;
  }

  // tgvmrioptimizer.cu:95-110
  void check_ready() const {
    if (with_op() && !op_) throw Error(PDT_ERR_STATE, "No operator is set!");
    if (!has_f_) throw Error(PDT_ERR_STATE, "No noisy data is set!");
  }

  // setInput0 extended with the second TGV primal: u = ubar = u0, v = vbar = v0 (two planes vx, vy),
  // p = q = 0.
  void set_input0_uv(const void* u0, const void* v0, const Dims& size, bool is_device, cudaStream_t st) {
    set_input0(u0, size, is_device, st);
    if (v0) {
      const size_t plane = plane_bytes();
      copy_in(field(F_VX, 0), v0, plane, is_device, st);
      copy_in(field(F_VY, 0), static_cast<const char*>(v0) + plane, plane, is_device, st);
      PDT_CUDA_CHECK(cudaMemcpyAsync(field(F_VBX, 0), field(F_VX, 0), plane, cudaMemcpyDeviceToDevice, st));
      PDT_CUDA_CHECK(cudaMemcpyAsync(field(F_VBY, 0), field(F_VY, 0), plane, cudaMemcpyDeviceToDevice, st));
    }
  }

  // One plane of the state (0..10), or with F_R the k-space dual r in the user's dense k-space layout.
  void get_field(int f, void* dst, bool is_device, cudaStream_t st) {
    if (!has_state_) throw Error(PDT_ERR_STATE, "There is no result yet!");
    if (f == F_R) {
      SolverHooks* hk = r_hooks(st);
      if (r_reset_ || r_.bytes != std::max<size_t>(hk->compact_elems(), 1) * sizeof(float2))
        throw Error(PDT_ERR_STATE, "There is no dual state yet: solve() first");
      const size_t bytes = numel_of(fsize_) * sizeof(float2);
      if (is_device) {
        hk->scatter(r_.as<float2>(), static_cast<float2*>(dst), st);
      } else {
        DevBuf tmp;
        tmp.ensure(std::max<size_t>(bytes, 1));
        hk->scatter(r_.as<float2>(), tmp.as<float2>(), st);
        PDT_CUDA_CHECK(cudaMemcpyAsync(dst, tmp.p, bytes, cudaMemcpyDeviceToHost, st));
        PDT_CUDA_CHECK(cudaStreamSynchronize(st));
      }
      return;
    }
    if (f < 0 || f >= F_COUNT) throw Error(PDT_ERR_INVALID_ARGUMENT, "unknown field");
    PDT_CUDA_CHECK(cudaMemcpyAsync(dst, field(f, parity_), plane_bytes(),
                                   is_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, st));
    if (!is_device) PDT_CUDA_CHECK(cudaStreamSynchronize(st));
  }

  // Replaces one plane of the state (0..10; a state must exist: setInput0 or a solve first), or with
  // F_R the k-space dual r from the user's dense k-space layout (entries on phase-encode lines the mask
  // never samples are not held: they never reach u). The next solve() continues from the new state.
  void set_field(int f, const void* src, bool is_device, cudaStream_t st) {
    if (f == F_R) {
      SolverHooks* hk = r_hooks(st);
      const size_t nk = hk->compact_elems();
      if (r_.bytes != std::max<size_t>(nk, 1) * sizeof(float2)) {
        r_.ensure(std::max<size_t>(nk, 1) * sizeof(float2));
        ++version_;
      }
      const size_t bytes = numel_of(fsize_) * sizeof(float2);
      if (is_device) {
        hk->gather(static_cast<const float2*>(src), r_.as<float2>(), st);
      } else {
        DevBuf tmp;
        tmp.ensure(std::max<size_t>(bytes, 1));
        PDT_CUDA_CHECK(cudaMemcpyAsync(tmp.p, src, bytes, cudaMemcpyHostToDevice, st));
        hk->gather(tmp.as<float2>(), r_.as<float2>(), st);
        PDT_CUDA_CHECK(cudaStreamSynchronize(st));
      }
      r_reset_ = false;
      return;
    }
    if (f < 0 || f >= F_COUNT) throw Error(PDT_ERR_INVALID_ARGUMENT, "unknown field");
    if (!has_state_) throw Error(PDT_ERR_STATE, "There is no state yet: setInput0 or solve() first");
    copy_in(field(f, parity_), src, plane_bytes(), is_device, st);
  }

  // Energy of the current primal state in FP64: out = {total, data term, first-order term, second-order term}.
  // TGV-MRI uses the final alpha of its continuation (alpha * reduction).
  void energy(cudaStream_t st, double out[4]) {
    check_ready();
    if (!has_state_) throw Error(PDT_ERR_STATE, "There is no result yet!");
    double a0 = params_.alpha0, a1 = params_.alpha1;
    if (kind_ == PDT_OPT_TGV_MRI) {
      a0 *= params_.reduction;
      a1 *= params_.reduction;
    }
    const bool has_v = tgv();
    double reg[2];
    reduce_regularizer(cplx_, field(F_U, parity_), has_v ? field(F_VX, parity_) : nullptr,
                       has_v ? field(F_VY, parity_) : nullptr, W_, H_, reg, st);
    double data;
    if (with_op()) {
      DevBuf ku;
      ku.ensure(std::max<size_t>(numel_of(fsize_) * sizeof(float2), 1));
      op_->forward(static_cast<const float2*>(field(F_U, parity_)), usize_, ku.as<float2>(), fsize_, st);
      // the with-operator r-prox (r + sigma (K u - f)) / (1 + sigma lambda) (tgv_kernels.cuh:213-223) is
      // the resolvent of F*(r) = <f, r> + lambda/2 |r|^2, i.e. F(z) = |z - f|^2 / (2 lambda)
      data = 0.5 * reduce_dist2(true, ku.p, f_.p, numel_of(fsize_), st);
      if (kind_ != PDT_OPT_TGV_MRI) data /= params_.lambda;
    } else {
      data = 0.5 * params_.lambda * reduce_dist2(cplx_, field(F_U, parity_), f_.p, (size_t)W_ * H_, st);
    }
    out[1] = data;
    if (has_v) {
      out[2] = a1 * reg[0];
      out[3] = a0 * reg[1];
    } else {
      out[2] = (kind_ == PDT_OPT_TV_OP || kind_ == PDT_OPT_TV) ? reg[0] : a1 * reg[0];
      out[3] = 0;
    }
    out[0] = out[1] + out[2] + out[3];
  }

  // Primal-dual gap and dual-constraint residuals (pdt_opt_gap). The compact k-space holds every row
  // of the sampled phase-encode lines; on the other lines r converges to -f, where primal and dual
  // terms are both |f|^2 / 2 and cancel in the gap.
  void gap(cudaStream_t st, double out[6]) {
    if (!with_op()) throw Error(PDT_ERR_INVALID_ARGUMENT, "the gap is defined for the with-operator optimizers");
    check_ready();
    if (!has_state_) throw Error(PDT_ERR_STATE, "There is no result yet!");
    SolverHooks* hk = op_->hooks();
    ensure_fc(hk, st);
    const size_t nk = hk->compact_elems();
    if (r_.bytes != std::max<size_t>(nk, 1) * sizeof(float2) || r_reset_)
      throw Error(PDT_ERR_STATE, "There is no dual state yet: solve() first");
    double e[4];
    energy(st, e);
    const double lam = kind_ == PDT_OPT_TGV_MRI ? 1.0 : params_.lambda;
    const double f_all = reduce_dist2(true, f_.p, nullptr, numel_of(fsize_), st);
    const double f_cmp = reduce_dist2(true, fc_.p, nullptr, nk, st);
    const double rr = reduce_dist2(true, r_.p, nullptr, nk, st);
    const double fr = reduce_dot_re(fc_.as<float2>(), r_.as<float2>(), nk, st);
    // -F*(r) = -<f, r> - lambda/2 |r|^2 on the stored lines; |f|^2 / (2 lambda) on the others (r = -f / lambda)
    const double dual = -fr - 0.5 * lam * rr + 0.5 * (f_all - f_cmp) / lam;
    DevBuf khr;
    khr.ensure((size_t)W_ * H_ * sizeof(float2));
    hk->adjoint_compact(r_.as<float2>(), khr.as<float2>(), st);
    const bool v = kind_ != PDT_OPT_TV_OP;
    double kkt[2];
    reduce_kkt(W_, H_, khr.as<float2>(), static_cast<const float2*>(field(F_PX, parity_)),
               static_cast<const float2*>(field(F_PY, parity_)),
               v ? static_cast<const float2*>(field(F_QXX, parity_)) : nullptr,
               v ? static_cast<const float2*>(field(F_QYY, parity_)) : nullptr,
               v ? static_cast<const float2*>(field(F_QXY, parity_)) : nullptr, kkt, st);
    out[0] = e[0] - dual;
    out[1] = e[0];
    out[2] = dual;
    out[3] = std::sqrt(kkt[0]);
    out[4] = std::sqrt(kkt[1]);
    out[5] = std::sqrt(reduce_dist2(true, khr.p, nullptr, (size_t)W_ * H_, st));
  }

  // A solve split in three: plan() enqueues the set-up on `st` and returns the per-iteration body,
  // the iterations run (graph replay or direct), finish() records the new state parity.
  struct Plan {
    int n = 0;     // calls of body
    int tail = 0;  // then calls of tail_body (parity continues)
    int iters = 0;  // primal-dual iterations in all (for the verbose report)
    int p0 = 0;
    uint64_t key = 0;
    bool verbose = false;
    std::function<void(int, cudaStream_t)> body, tail_body;
  };

  Plan plan(bool verbose, cudaStream_t st) {
    check_ready();
    return with_op() ? plan_with_op(verbose, st) : plan_denoise(verbose, st);
  }
  void finish(const Plan& p) {
    parity_ = p.p0 ^ ((p.n + p.tail) & 1);
    if (p.verbose && !with_op()) print_iters(p.iters ? p.iters : p.n);
  }
  void solve(bool verbose, cudaStream_t st) {
    Plan p = plan(verbose, st);
    run_iterations(graph_, p.key, p.n, profiling_ ? p.n + 2 : kGraphIters, p.body, st, capture_stream());
    for (int i = 0; i < p.tail; ++i) p.tail_body((p.n + i) & 1, st);
    finish(p);
  }
  const OpImpl* op_ptr() const { return op_.get(); }
  // Tells the operator that its rounds launch beside other problems' kernels (SolverHooks::set_concurrent).
  void set_concurrent(bool on) {
    if (op_)
      if (SolverHooks* hk = op_->hooks()) hk->set_concurrent(on);
  }

  Dims result_size() const {
    if (!has_state_) throw Error(PDT_ERR_STATE, "There is no result yet!");
    return usize_;
  }
  // Reads and clears the with-operator solvers' non-finite flag (word 2 of the alpha table's header, set
  // by the primal kernel when a new u or v is NaN or infinite); throws PDT_ERR_NUMERIC if it was set.
  // Waits for `st`. The reference has no such check (its solve loop only checks launches,
  // tgvmrioptimizer.cu:163-198).
  void check_numeric(cudaStream_t st) {
    if (!with_op() || !alpha_.p) return;
    int* w = alpha_.as<int>() + 2;
    int flag = 0;
    PDT_CUDA_CHECK(cudaMemcpyAsync(&flag, w, sizeof(int), cudaMemcpyDeviceToHost, st));
    PDT_CUDA_CHECK(cudaStreamSynchronize(st));
    if (!flag) return;
    PDT_CUDA_CHECK(cudaMemsetAsync(w, 0, sizeof(int), st));
    PDT_CUDA_CHECK(cudaStreamSynchronize(st));
    throw Error(PDT_ERR_NUMERIC, "Non-finite values (NaN or Inf) appeared in the primal variables: check the noisy "
                                 "data, the operator's constants and the parameters");
  }

  // Everything the solve's kernels report on the device: a bounded wait of the operator's kernels that
  // gave up (PDT_ERR_TIMEOUT) first, then the non-finite flag (PDT_ERR_NUMERIC). Waits for `st`.
  void check_device(cudaStream_t st) {
    PDT_CUDA_CHECK(cudaStreamSynchronize(st));
    if (op_) op_->check_device_errors();
    check_numeric(st);
  }

  void get_result(void* dst, bool is_device, cudaStream_t st) {
    if (!has_state_) throw Error(PDT_ERR_STATE, "There is no result yet!");
    const size_t bytes = plane_bytes();
    PDT_CUDA_CHECK(cudaMemcpyAsync(dst, field(F_U, parity_), bytes,
                                   is_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, st));
    if (!is_device) PDT_CUDA_CHECK(cudaStreamSynchronize(st));
  }

  // Runs `iters` further iterations launch by launch with a CUDA event after each phase and returns the
  // mean duration of every phase in ms (the iterations advance the solver state like solve() does).
  void profile(int iters, cudaStream_t st, std::vector<std::string>& names, std::vector<double>& ms) {
    if (!has_state_) throw Error(PDT_ERR_STATE, "There is no result yet!");
    struct Marker : PhaseMarker {
      std::vector<cudaEvent_t> ev;
      std::vector<std::string> nm;
      void mark(const char* phase, cudaStream_t s) override {
        cudaEvent_t e;
        PDT_CUDA_CHECK(cudaEventCreate(&e));
        PDT_CUDA_CHECK(cudaEventRecord(e, s));
        ev.push_back(e);
        nm.push_back(phase);
      }
      ~Marker() {
        for (auto e : ev) cudaEventDestroy(e);
      }
    } mk;
    mk.mark("start", st);
    prof_ = &mk;
    const uint32_t saved = params_.max_iter;
    try {
      params_.max_iter = (uint32_t)iters - 1;
      profiling_ = true;
      solve(false, st);
    } catch (...) {
      profiling_ = false;
      params_.max_iter = saved;
      prof_ = nullptr;
      throw;
    }
    profiling_ = false;
    params_.max_iter = saved;
    prof_ = nullptr;
    PDT_CUDA_CHECK(cudaStreamSynchronize(st));
    names.clear();
    ms.clear();
    std::map<std::string, size_t> slot;
    for (size_t i = 1; i < mk.ev.size(); ++i) {
      float t = 0;
      PDT_CUDA_CHECK(cudaEventElapsedTime(&t, mk.ev[i - 1], mk.ev[i]));
      auto it = slot.find(mk.nm[i]);
      if (it == slot.end()) {
        slot[mk.nm[i]] = names.size();
        names.push_back(mk.nm[i]);
        ms.push_back(t);
      } else {
        ms[it->second] += t;
      }
    }
    for (auto& v : ms) v /= iters;
  }

  // The operator hooks that hold r, after the checks a k-space dual needs.
  SolverHooks* r_hooks(cudaStream_t st) {
    if (!with_op()) throw Error(PDT_ERR_INVALID_ARGUMENT, "only the with-operator optimizers have a k-space dual");
    check_ready();
    SolverHooks* hk = op_->hooks();
    ensure_fc(hk, st);
    return hk;
  }

  // Streams are created on first use so that handles can be made (and misused) without a device.
  cudaStream_t own_stream() {
    if (!own_) PDT_CUDA_CHECK(cudaStreamCreateWithFlags(&own_, cudaStreamNonBlocking));
    return own_;
  }
  cudaStream_t capture_stream() {
    if (!cap_) PDT_CUDA_CHECK(cudaStreamCreateWithFlags(&cap_, cudaStreamNonBlocking));
    return cap_;
  }
  // side stream and fork/join events of the concurrent dual update
  void ensure_aux() {
    if (!aux_) PDT_CUDA_CHECK(cudaStreamCreateWithFlags(&aux_, cudaStreamNonBlocking));
    if (!ev_fork_) PDT_CUDA_CHECK(cudaEventCreateWithFlags(&ev_fork_, cudaEventDisableTiming));
    if (!ev_join_) PDT_CUDA_CHECK(cudaEventCreateWithFlags(&ev_join_, cudaEventDisableTiming));
  }

 private:
  static void copy_in(void* dst, const void* src, size_t bytes, bool is_device, cudaStream_t st) {
    if (!bytes) return;
    PDT_CUDA_CHECK(cudaMemcpyAsync(dst, src, bytes, is_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st));
    if (!is_device) PDT_CUDA_CHECK(cudaStreamSynchronize(st));
  }

  size_t plane_bytes() const { return (size_t)W_ * H_ * pix(); }
  // Fields that are read at neighbouring pixels ping-pong between two copies; in the primal-first TGV
  // denoising order u, v do too.
  bool pingpong(int f) const {
    // the denoising kernels read u (and v) at neighbouring pixels (the TV kernel through its halo)
    if (f == F_U || f == F_VX || f == F_VY) return kind_ == PDT_OPT_TGV || kind_ == PDT_OPT_TV;
    return true;
  }
  void* field(int f, int set) const {
    const int s = pingpong(f) ? set : 0;
    return static_cast<char*>(img_.p) + ((size_t)s * F_COUNT + f) * plane_bytes();
  }
  ImgPtrs ptrs(int set) const {
    ImgPtrs p;
    p.u = field(F_U, set);
    p.ub = field(F_UB, set);
    p.vx = field(F_VX, set);
    p.vy = field(F_VY, set);
    p.vbx = field(F_VBX, set);
    p.vby = field(F_VBY, set);
    p.px = field(F_PX, set);
    p.py = field(F_PY, set);
    p.qxx = field(F_QXX, set);
    p.qyy = field(F_QYY, set);
    p.qxy = field(F_QXY, set);
    return p;
  }
  void alloc_state(const Dims& size) {
    if (size != usize_ || !img_.p) {
      usize_ = size;
      W_ = (int)size[0];
      H_ = (int)size[1];
      img_.ensure(std::max<size_t>(2 * F_COUNT * plane_bytes(), 1));
      ++version_;
    }
  }

  void print_params() const {
    std::ostringstream os;
    if (kind_ == PDT_OPT_TGV_MRI) {
      os << "TgvMriParameters:\n alpha0=" << (float)params_.alpha0 << "\n alpha1=" << (float)params_.alpha1
         << "\n check=" << params_.check << "\n reduction=" << (float)params_.reduction
         << "\n max_iter=" << params_.max_iter << "\n";
    } else if (tgv()) {
      os << "TgvParameters:\n check=" << params_.check << "\n lambda=" << (float)params_.lambda
         << "\n alpha0=" << (float)params_.alpha0 << "\n alpha1=" << (float)params_.alpha1
         << "\n max_iter=" << params_.max_iter << "\n";
    } else {
      os << "TvParameters:\n check=" << params_.check << "\n lambda=" << (float)params_.lambda
         << "\n max_iter=" << params_.max_iter << "\n";
    }
    std::cout << os.str() << std::endl;
  }

  // TvOptimizer::solve (tvoptimizer.cu:76-125) / TgvOptimizer::solve (tgvoptimizer.cu:80-141).
  Plan plan_denoise(bool verbose, cudaStream_t st) {
    if (!has_state_) {
      if (verbose) std::cout << "Initialization with f" << std::endl;
      set_input0(f_.p, fsize_, true, st);
    }
    size_check_eq(usize_, fsize_);
    const bool is_tgv = kind_ == PDT_OPT_TGV;
    const float tau = (float)(1.0 / std::sqrt(is_tgv ? 12.0 : 8.0));
    const float sigma = tau;
    const float lambda = (float)params_.lambda;
    const float a0 = (float)params_.alpha0, a1 = (float)params_.alpha1;
    if (verbose) print_params();
    Plan pl;
    pl.iters = (int)params_.max_iter + 1;
    pl.n = pl.iters;
    pl.p0 = parity_;
    pl.verbose = verbose;
    const int p0 = parity_;
    if (is_tgv) {
      pl.body = [=](int par, cudaStream_t s) {
        const int in = p0 ^ par, out = in ^ 1;
        launch_tgv_denoise_step(cplx_, W_, H_, ptrs(in), ptrs(out), f_.p, tau, sigma, lambda, a0, a1, s);
        if (prof_) prof_->mark("tgv_denoise_step", s);
      };
    } else if (!tv_multi_faster(tau, sigma, lambda, st)) {
      pl.body = [=](int par, cudaStream_t s) {
        const int in = p0 ^ par, out = in ^ 1;
        launch_tv_step(cplx_, W_, H_, ptrs(in), ptrs(out), f_.p, tau, sigma, lambda, s);
        if (prof_) prof_->mark("tv_step", s);
      };
    } else {
      // kTvStepsPerLaunch iterations per launch, then the remainder one at a time
      pl.n = pl.iters / kTvStepsPerLaunch;
      pl.tail = pl.iters % kTvStepsPerLaunch;
      pl.body = [=](int par, cudaStream_t s) {
        const int in = p0 ^ par, out = in ^ 1;
        launch_tv_multi_step(cplx_, W_, H_, ptrs(in), ptrs(out), f_.p, tau, sigma, lambda, s);
        if (prof_) prof_->mark("tv_multi_step", s);
      };
      pl.tail_body = [=](int par, cudaStream_t s) {
        const int in = p0 ^ par, out = in ^ 1;
        launch_tv_step(cplx_, W_, H_, ptrs(in), ptrs(out), f_.p, tau, sigma, lambda, s);
        if (prof_) prof_->mark("tv_step", s);
      };
    }
    pl.key = graph_key({(uintptr_t)img_.p, (uintptr_t)f_.p, (uintptr_t)W_, (uintptr_t)H_, (uintptr_t)p0,
                        (uintptr_t)cplx_, fbits(lambda), fbits(a0), fbits(a1)});
    return pl;
  }

  // TV denoising runs kTvStepsPerLaunch iterations per launch (temporal blocking in shared memory, the
  // faster choice while the state stays in L2) or one per launch (for large images the halo recompute can
  // cost more than the DRAM passes it saves). Images of at least 2^20 pixels time both once per
  // (W, H, pixel type) on zeroed scratch state -- 2 x 4 iterations against 8, best of two -- and the
  // choice is kept for the process.
  bool tv_multi_faster(float tau, float sigma, float lambda, cudaStream_t st) {
    if ((size_t)W_ * H_ < ((size_t)1 << 20)) return true;
    static std::mutex mu;
    static std::map<std::tuple<int, int, bool>, bool> cache;
    const auto key = std::make_tuple(W_, H_, cplx_);
    std::lock_guard<std::mutex> lock(mu);
    auto hit = cache.find(key);
    if (hit != cache.end()) return hit->second;
    DevBuf scratch;
    scratch.ensure(img_.bytes);
    PDT_CUDA_CHECK(cudaMemsetAsync(scratch.p, 0, scratch.bytes, st));
    auto sp = [&](int set) {
      ImgPtrs p = ptrs(set);
      const ptrdiff_t shift = static_cast<char*>(scratch.p) - static_cast<char*>(img_.p);
      for (void** q : {&p.u, &p.ub, &p.vx, &p.vy, &p.vbx, &p.vby, &p.px, &p.py, &p.qxx, &p.qyy, &p.qxy})
        *q = static_cast<char*>(*q) + shift;
      return p;
    };
    const uint64_t launches0 = g_launches.load();
    cudaEvent_t e0, e1, e2;
    PDT_CUDA_CHECK(cudaEventCreate(&e0));
    PDT_CUDA_CHECK(cudaEventCreate(&e1));
    PDT_CUDA_CHECK(cudaEventCreate(&e2));
    float best_multi = 1e30f, best_single = 1e30f;
    for (int rep = 0; rep < 2; ++rep) {
      PDT_CUDA_CHECK(cudaEventRecord(e0, st));
      for (int i = 0; i < 2; ++i) launch_tv_multi_step(cplx_, W_, H_, sp(i & 1), sp((i & 1) ^ 1), f_.p, tau, sigma, lambda, st);
      PDT_CUDA_CHECK(cudaEventRecord(e1, st));
      for (int i = 0; i < 2 * kTvStepsPerLaunch; ++i)
        launch_tv_step(cplx_, W_, H_, sp(i & 1), sp((i & 1) ^ 1), f_.p, tau, sigma, lambda, st);
      PDT_CUDA_CHECK(cudaEventRecord(e2, st));
      PDT_CUDA_CHECK(cudaEventSynchronize(e2));
      float m = 0, g = 0;
      PDT_CUDA_CHECK(cudaEventElapsedTime(&m, e0, e1));
      PDT_CUDA_CHECK(cudaEventElapsedTime(&g, e1, e2));
      best_multi = std::min(best_multi, m);
      best_single = std::min(best_single, g);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaEventDestroy(e2);
    g_launches.fetch_sub(g_launches.load() - launches0);  // tuning launches are not solver work
    return cache[key] = best_multi <= best_single;
  }

  // TgvMriOptimizer::solve (tgvmrioptimizer.cu:93-203), TgvOptimizerWithOp::solve
  // (tgvoptimizerwithop.cu:89-179), TvOptimizerWithOp::solve (tvoptimizerwithop.cu:86-164).
  Plan plan_with_op(bool verbose, cudaStream_t st) {
    SolverHooks* hk = op_->hooks();
    if (!has_state_) {
      if (verbose) std::cout << "Initialization with A^T(f)" << std::endl;
      const Dims in = op_->input_size(fsize_);
      op_->operator_check(in, fsize_);
      alloc_state(in);
      ensure_fc(hk, st);
      PDT_CUDA_CHECK(cudaMemsetAsync(img_.p, 0, img_.bytes, st));
      parity_ = 0;
      hk->adjoint_compact(fc_.as<float2>(), static_cast<float2*>(field(F_U, 0)), st);
      PDT_CUDA_CHECK(cudaMemcpyAsync(field(F_UB, 0), field(F_U, 0), plane_bytes(), cudaMemcpyDeviceToDevice, st));
      has_state_ = true;
    }
    op_->operator_check(usize_, fsize_);
    ensure_fc(hk, st);
    const size_t nk = hk->compact_elems();
    if (r_.bytes != std::max<size_t>(nk, 1) * sizeof(float2)) {
      r_.ensure(std::max<size_t>(nk, 1) * sizeof(float2));
      r_reset_ = true;
      ++version_;
    }
    if (r_reset_) {
      PDT_CUDA_CHECK(cudaMemsetAsync(r_.p, 0, r_.bytes, st));
      r_reset_ = false;
    }
    const int G = hk->groups();
    const long long gstride = hk->group_stride();
    const size_t khr_bytes = (size_t)G * gstride * sizeof(float2);
    if (khr_.bytes != khr_bytes) {
      khr_.ensure(khr_bytes);
      ++version_;
    }
    // step sizes (tgvmrioptimizer.cu:132-134; *withop.cu: tau = sigma = 1/8)
    float tau = kind_ == PDT_OPT_TGV_MRI ? 1.0f / 16.0f : 1.0f / 8.0f;
    float sigma = 1.0f / 8.0f;
    if (step_tau_ > 0.f) tau = step_tau_;  // pdt_opt_set_steps (no reference counterpart)
    if (step_sigma_ > 0.f) sigma = step_sigma_;
    const float lambda = kind_ == PDT_OPT_TGV_MRI ? 1.0f : (float)params_.lambda;
    // alpha table for every iteration (tgvmrioptimizer.cu:144-155 in real_type)
    const unsigned K = params_.max_iter;
    const int n = (int)K + 1;
    std::vector<float> tab(2 * (size_t)n);
    for (unsigned k = 0; k <= K; ++k) {
      float a0 = (float)params_.alpha0, a1 = (float)params_.alpha1;
      if (kind_ == PDT_OPT_TGV_MRI) alpha_at(k, a0, a1);
      tab[2 * k] = a0;
      tab[2 * k + 1] = a1;
    }
    if (verbose) {
      print_params();
      for (unsigned k = 0; k <= K; ++k)
        if (params_.check && !(k % params_.check)) {
          if (kind_ == PDT_OPT_TGV_MRI)
            std::cout << "iter=" << k << " alpha0=" << tab[2 * k] << " alpha1=" << tab[2 * k + 1] << std::endl;
          else
            std::cout << "iter=" << k << " lambda=" << lambda << std::endl;
        }
    }
    // device layout: a 64-byte header {iteration counter, table length n} at a fixed offset, then the
    // table. Graph kernels keep the header's address, so it must not move when n changes.
    alpha_.ensure(kAlphaHeader + tab.size() * sizeof(float));
    int* iter = alpha_.as<int>();
    if (alpha_host_ != tab) {
      std::vector<char> img(alpha_.bytes, 0);
      const int hdr[2] = {-1, n};
      std::memcpy(img.data(), hdr, sizeof(hdr));
      std::memcpy(img.data() + kAlphaHeader, tab.data(), tab.size() * sizeof(float));
      PDT_CUDA_CHECK(cudaMemcpyAsync(alpha_.p, img.data(), img.size(), cudaMemcpyHostToDevice, st));
      PDT_CUDA_CHECK(cudaStreamSynchronize(st));
      alpha_host_ = tab;
    }
    PDT_CUDA_CHECK(cudaMemsetAsync(iter, 0, sizeof(int), st));  // the primal kernel advances it
    const bool is_tgv = kind_ != PDT_OPT_TV_OP;
    const int p0 = parity_;
    const float* atab = reinterpret_cast<const float*>(alpha_.as<char>() + kAlphaHeader);
    float2* khr = khr_.as<float2>();
    Plan pl;
    pl.n = n;
    pl.p0 = p0;
    pl.verbose = verbose;
    ensure_aux();
    cudaStream_t aux = aux_;
    cudaEvent_t ev_fork = ev_fork_, ev_join = ev_join_;
    // one iteration: the dual update runs inside the operator's round where the operator has idle
    // blocks for it (profiling then times it as part of that launch), else on `aux`, forked from and
    // joined back into `s`, concurrently with the round (profiling runs it in line so that every phase
    // has its own interval)
    const bool fused = hk->can_fuse_dual(W_, H_);
    pl.body = [=](int par, cudaStream_t s) {
      const int in = p0 ^ par, out = in ^ 1;
      const float2* ubar = static_cast<const float2*>(field(F_UB, in));
      if (fused) {
        const DualStep ds{ptrs(in), ptrs(out), sigma, atab, iter, W_, H_, is_tgv ? 1 : 0};
        hk->round(ubar, r_.as<float2>(), fc_.as<float2>(), sigma, lambda, khr, nullptr, s, prof_, &ds);
      } else if (prof_) {
        launch_mri_dual(is_tgv, W_, H_, ptrs(in), ptrs(out), sigma, atab, iter, s);
        prof_->mark(is_tgv ? "mri_dual_tgv" : "mri_dual_tv", s);
        hk->round(ubar, r_.as<float2>(), fc_.as<float2>(), sigma, lambda, khr, nullptr, s, prof_);
      } else {
        PDT_CUDA_CHECK(cudaEventRecord(ev_fork, s));
        PDT_CUDA_CHECK(cudaStreamWaitEvent(aux, ev_fork, 0));
        launch_mri_dual(is_tgv, W_, H_, ptrs(in), ptrs(out), sigma, atab, iter, aux);
        PDT_CUDA_CHECK(cudaEventRecord(ev_join, aux));
        hk->round(ubar, r_.as<float2>(), fc_.as<float2>(), sigma, lambda, khr, nullptr, s, nullptr);
        PDT_CUDA_CHECK(cudaStreamWaitEvent(s, ev_join, 0));
      }
      launch_mri_primal(is_tgv, W_, H_, ptrs(out), khr, G, gstride, tau, iter, s);
      if (prof_) prof_->mark(is_tgv ? "mri_primal_tgv" : "mri_primal_tv", s);
    };
    pl.key = graph_key({(uintptr_t)img_.p, (uintptr_t)r_.p, (uintptr_t)fc_.p, (uintptr_t)khr_.p,
                        (uintptr_t)alpha_.p, (uintptr_t)alpha_.bytes, (uintptr_t)op_.get(),
                        (uintptr_t)op_->generation(), (uintptr_t)W_, (uintptr_t)H_, (uintptr_t)G, (uintptr_t)p0,
                        (uintptr_t)is_tgv, (uintptr_t)fused, fbits(lambda), fbits(tau), fbits(sigma),
                        (uintptr_t)version_});
    return pl;
  }

  void ensure_fc(SolverHooks* hk, cudaStream_t st) {
    if (op_gen_ != op_->generation()) {  // new constants: the compact layout may have changed
      op_gen_ = op_->generation();
      fc_valid_ = false;
    }
    if (fc_valid_) return;
    const size_t nk = hk->compact_elems();
    fc_.ensure(std::max<size_t>(nk, 1) * sizeof(float2));
    hk->gather(f_.as<float2>(), fc_.as<float2>(), st);
    fc_valid_ = true;
    ++version_;
  }

  // alpha_k = exp(k/K log(alpha*reduction) + (K-k)/K log(alpha)) in float (tgvmrioptimizer.cu:120-155).
  void alpha_at(unsigned k, float& a0, float& a1) const {
    const float a00 = (float)params_.alpha0, a10 = (float)params_.alpha1;
    const float red = (float)params_.reduction;
    const float a01 = a00 * red, a11 = a10 * red;
    if (params_.max_iter == 0) {  // the reference divides 0/0 here; use the k/K -> 0 limit
      a0 = a00;
      a1 = a10;
      return;
    }
    const float dmax = (float)params_.max_iter, dk = (float)k;
    a0 = std::exp(dk / dmax * std::log(a01) + (dmax - dk) / dmax * std::log(a00));
    a1 = std::exp(dk / dmax * std::log(a11) + (dmax - dk) / dmax * std::log(a10));
  }

  void print_iters(int n) const {
    for (int k = 0; k < n; ++k)
      if (params_.check && !(k % params_.check)) std::cout << "iter=" << k << std::endl;
  }

  // Identity of a captured iteration graph: every pointer and scalar baked into its kernel nodes.
 public:
  static uintptr_t fbits(float v) {
    uint32_t b;
    std::memcpy(&b, &v, 4);
    return b;
  }
  static uint64_t graph_key(std::initializer_list<uintptr_t> vals) {
    uint64_t h = 1469598103934665603ull;
    for (uintptr_t v : vals) h = (h ^ (uint64_t)v) * 0x100000001b3ull;
    return h;
  }

 private:

  static constexpr int kGraphIters = 20;
  static constexpr size_t kAlphaHeader = 64;

  pdt_opt_kind kind_;
  bool cplx_;
  std::shared_ptr<OpImpl> op_;
  DevBuf f_;
  Dims fsize_;
  bool has_f_ = false;
  bool has_state_ = false;
  Dims usize_;
  int W_ = 0, H_ = 0;
  int parity_ = 0;
  DevBuf img_, r_, fc_, khr_, alpha_;
  std::vector<float> alpha_host_;
  bool r_reset_ = true, fc_valid_ = false;
  uint64_t op_gen_ = 0;
  uint64_t version_ = 1;
  IterGraph graph_;
  PhaseMarker* prof_ = nullptr;
  bool profiling_ = false;
  cudaStream_t own_ = nullptr, cap_ = nullptr, aux_ = nullptr;
  cudaEvent_t ev_fork_ = nullptr, ev_join_ = nullptr;
};


// ------------------------------------------------------------------------------------------------
// Batched solve: independent reconstructions advance together. Every problem's iteration body runs on
// its own branch of one captured CUDA graph (forked worker streams), so the small kernels of many
// problems execute concurrently and fill the GPU; chunks of kBatchIters iterations replay the graph.
// ------------------------------------------------------------------------------------------------
class BatchImpl {
 public:
  ~BatchImpl() {
    graph_.reset();
    for (auto s : workers_) cudaStreamDestroy(s);
    for (auto e : events_) cudaEventDestroy(e);
    if (cap_) cudaStreamDestroy(cap_);
  }
  void add(OptImpl* o) {
    if (o->op_ptr())
      for (OptImpl* q : opts_)
        if (q->op_ptr() == o->op_ptr())
          throw Error(PDT_ERR_INVALID_ARGUMENT, "optimizers in one batch need distinct operators (an operator's "
                                                "scratch serves one solve at a time)");
    for (OptImpl* q : opts_)
      if (q == o) throw Error(PDT_ERR_INVALID_ARGUMENT, "optimizer already in the batch");
    opts_.push_back(o);
  }
  size_t size() const { return opts_.size(); }
  // Raises the first problem's device report (and clears every problem's).
  void check_device(cudaStream_t st) {
    std::string first;
    pdt_status code = PDT_OK;
    for (OptImpl* o : opts_) try {
        o->check_device(st);
      } catch (const Error& e) {
        if (first.empty()) first = e.what(), code = e.code;
      }
    if (!first.empty()) throw Error(code, first);
  }

  void solve(bool verbose, cudaStream_t st) {
    if (opts_.empty()) return;
    // every round of the batch runs beside the other problems' launches
    struct Concurrent {
      std::vector<OptImpl*>& opts;
      explicit Concurrent(std::vector<OptImpl*>& o) : opts(o) {
        for (OptImpl* q : opts) q->set_concurrent(true);
      }
      ~Concurrent() {
        for (OptImpl* q : opts) q->set_concurrent(false);
      }
    } concurrent(opts_);
    std::vector<OptImpl::Plan> plans;
    plans.reserve(opts_.size());
    for (OptImpl* o : opts_) plans.push_back(o->plan(verbose, st));
    ensure_streams();
    int nmin = plans[0].n;
    uint64_t key = 7;
    for (auto& p : plans) {
      nmin = std::min(nmin, p.n);
      key = OptImpl::graph_key({(uintptr_t)key, (uintptr_t)p.key});
    }
    const int full = nmin / kBatchIters;
    if (full > 0) {
      if (!graph_.exec || graph_.key != key) {
        graph_.reset();
        const uint64_t before = g_launches.load();
        PDT_CUDA_CHECK(cudaStreamBeginCapture(cap_, cudaStreamCaptureModeThreadLocal));
        try {
          fork_join(cap_, [&](size_t i, cudaStream_t w) {
            for (int it = 0; it < kBatchIters; ++it) plans[i].body(it & 1, w);
          });
        } catch (...) {
          cudaGraph_t dummy = nullptr;
          cudaStreamEndCapture(cap_, &dummy);
          if (dummy) cudaGraphDestroy(dummy);
          throw;
        }
        cudaGraph_t graph = nullptr;
        PDT_CUDA_CHECK(cudaStreamEndCapture(cap_, &graph));
        graph_.kernels = g_launches.load() - before;
        g_launches.fetch_sub(graph_.kernels);
        cudaError_t e = cudaGraphInstantiate(&graph_.exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) throw Error(PDT_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
        graph_.key = key;
      }
      for (int i = 0; i < full; ++i) {
        PDT_CUDA_CHECK(cudaGraphLaunch(graph_.exec, st));
        count_launch(graph_.kernels);
      }
    }
    // remaining iterations of every problem (uneven max_iter), concurrently
    fork_join(st, [&](size_t i, cudaStream_t w) {
      for (int it = full * kBatchIters; it < plans[i].n; ++it) plans[i].body(it & 1, w);
      for (int t = 0; t < plans[i].tail; ++t) plans[i].tail_body((plans[i].n + t) & 1, w);
    });
    for (size_t i = 0; i < opts_.size(); ++i) opts_[i]->finish(plans[i]);
  }

 private:
  static constexpr int kBatchIters = 10;  // even: every replay returns each problem to its parity
  static constexpr int kMaxStreams = 32;

  // Worker streams: one per problem up to kMaxStreams (PDT_BATCH_STREAMS overrides, 1 .. 128). With more
  // problems than streams, problems go to streams longest first, each to the stream with the least work
  // so far (the graph's critical path is the most loaded stream).
  void ensure_streams() {
    static const int env_streams = [] {
      const char* e = std::getenv("PDT_BATCH_STREAMS");
      return (e && *e) ? std::max(1, std::min(128, std::atoi(e))) : kMaxStreams;
    }();
    const size_t want = std::min<size_t>(opts_.size(), (size_t)env_streams);
    if (!cap_) PDT_CUDA_CHECK(cudaStreamCreateWithFlags(&cap_, cudaStreamNonBlocking));
    while (workers_.size() < want) {
      cudaStream_t s;
      PDT_CUDA_CHECK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
      workers_.push_back(s);
    }
    while (events_.size() < workers_.size() + 1) {
      cudaEvent_t e;
      PDT_CUDA_CHECK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
      events_.push_back(e);
    }
    const size_t P = std::min(want, workers_.size());
    std::vector<size_t> cost(opts_.size());
    for (size_t i = 0; i < cost.size(); ++i) cost[i] = opts_[i]->work_estimate();
    owner_ = assign_longest_first(cost, P);
    nworkers_ = P;
  }
  // Runs fn(problem, worker stream) for every problem on worker streams forked from and joined back into `on`.
  template <class F>
  void fork_join(cudaStream_t on, F&& fn) {
    const size_t P = nworkers_;
    PDT_CUDA_CHECK(cudaEventRecord(events_[0], on));
    for (size_t w = 0; w < P; ++w) PDT_CUDA_CHECK(cudaStreamWaitEvent(workers_[w], events_[0], 0));
    for (size_t i = 0; i < opts_.size(); ++i) fn(i, workers_[owner_[i]]);
    for (size_t w = 0; w < P; ++w) {
      PDT_CUDA_CHECK(cudaEventRecord(events_[w + 1], workers_[w]));
      PDT_CUDA_CHECK(cudaStreamWaitEvent(on, events_[w + 1], 0));
    }
  }

  std::vector<OptImpl*> opts_;
  std::vector<cudaStream_t> workers_;
  std::vector<cudaEvent_t> events_;
  std::vector<size_t> owner_;  // worker stream of each problem
  size_t nworkers_ = 0;
  cudaStream_t cap_ = nullptr;
  IterGraph graph_;
};

}  // namespace pdt

// ==================================================================================================
// C ABI
// ==================================================================================================
using namespace pdt;

struct pdt_op {
  std::shared_ptr<OpImpl> impl;
};
struct pdt_opt {
  std::unique_ptr<OptImpl> impl;
};
struct pdt_batch {
  std::unique_ptr<BatchImpl> impl;
};

static thread_local std::string t_last_error;

void pdt::set_last_error(const std::string& msg) { t_last_error = msg; }

template <class F>
static pdt_status guarded(F&& fn) {
  try {
    fn();
    return PDT_OK;
  } catch (const Error& e) {
    t_last_error = e.what();
    return e.code;
  } catch (const std::bad_alloc&) {
    t_last_error = "host allocation failed";
    return PDT_ERR_ALLOC;
  } catch (const std::exception& e) {
    t_last_error = e.what();
    return PDT_ERR_INVALID_ARGUMENT;
  }
}

static Dims dims_in(int ndim, const int64_t* size) {
  if (ndim < 1 || ndim > 4 || !size) throw Error(PDT_ERR_INVALID_ARGUMENT, "bad ndim or null size");
  Dims d(size, size + ndim);
  for (auto v : d)
    if (v < 0) throw Error(PDT_ERR_INVALID_ARGUMENT, "negative size");
  return d;
}

template <class T>
static T* need(T* p, const char* what) {
  if (!p) throw Error(PDT_ERR_INVALID_ARGUMENT, std::string("null ") + what);
  return p;
}

// Device staging for host-pointer calls.
static void* dev_copy_of(const void* host, size_t bytes, DevBuf& buf, cudaStream_t st) {
  buf.ensure(std::max<size_t>(bytes, 1));
  if (bytes) PDT_CUDA_CHECK(cudaMemcpyAsync(buf.p, host, bytes, cudaMemcpyHostToDevice, st));
  return buf.p;
}

extern "C" {

const char* pdt_last_error(void) { return t_last_error.c_str(); }
int pdt_version(void) { return 1; }
uint64_t pdt_launch_count(void) { return g_launches.load(); }

pdt_status pdt_host_alloc(size_t bytes, void** out) {
  return guarded([&] {
    need(out, "out");
    cudaError_t e = cudaMallocHost(out, std::max<size_t>(bytes, 1));
    if (e != cudaSuccess) throw Error(PDT_ERR_ALLOC, std::string("cudaMallocHost: ") + cudaGetErrorString(e));
  });
}
pdt_status pdt_host_free(void* p) {
  return guarded([&] {
    if (p) PDT_CUDA_CHECK(cudaFreeHost(p));
  });
}
pdt_status pdt_stream_synchronize(void* stream) {
  return guarded([&] { PDT_CUDA_CHECK(cudaStreamSynchronize(static_cast<cudaStream_t>(stream))); });
}

pdt_status pdt_op_create(pdt_op_kind kind, const pdt_kv* cfg, int ncfg, pdt_op** out) {
  return guarded([&] {
    need(out, "out");
    if (ncfg < 0 || (ncfg > 0 && !cfg)) throw Error(PDT_ERR_INVALID_ARGUMENT, "bad config array");
    auto h = std::make_unique<pdt_op>();
    h->impl = make_operator(kind, to_map(cfg, ncfg));
    *out = h.release();
  });
}

pdt_status pdt_op_destroy(pdt_op* op) {
  return guarded([&] { delete op; });
}

pdt_status pdt_op_add_constant(pdt_op* op, pdt_dtype dtype, int ndim, const int64_t* size, const void* data,
                               int is_device) {
  return guarded([&] {
    need(op, "operator");
    if (dtype != PDT_F32 && dtype != PDT_C64) throw Error(PDT_ERR_INVALID_ARGUMENT, "bad dtype");
    const Dims d = dims_in(ndim, size);
    if (numel_of(d)) need(data, "data");
    op->impl->add_constant(dtype, d, data, is_device != 0);
  });
}

pdt_status pdt_op_replace_constant(pdt_op* op, int idx, pdt_dtype dtype, int ndim, const int64_t* size,
                                   const void* data, int is_device, void* stream) {
  return guarded([&] {
    need(op, "operator");
    if (dtype != PDT_F32 && dtype != PDT_C64) throw Error(PDT_ERR_INVALID_ARGUMENT, "bad dtype");
    if (idx < 0) throw Error(PDT_ERR_INVALID_ARGUMENT, "negative constant index");
    const Dims d = dims_in(ndim, size);
    if (numel_of(d)) need(data, "data");
    op->impl->replace_constant((unsigned)idx, dtype, d, data, is_device != 0, static_cast<cudaStream_t>(stream));
    if (!stream) PDT_CUDA_CHECK(cudaStreamSynchronize(nullptr));
  });
}

pdt_status pdt_op_input_size(pdt_op* op, int out_ndim, const int64_t* out_size, int* in_ndim, int64_t* in_size) {
  return guarded([&] {
    need(op, "operator");
    need(in_ndim, "in_ndim");
    need(in_size, "in_size");
    const Dims r = op->impl->input_size(dims_in(out_ndim, out_size));
    *in_ndim = (int)r.size();
    for (size_t i = 0; i < r.size(); ++i) in_size[i] = r[i];
  });
}

pdt_status pdt_op_output_size(pdt_op* op, int in_ndim, const int64_t* in_size, int* out_ndim, int64_t* out_size) {
  return guarded([&] {
    need(op, "operator");
    need(out_ndim, "out_ndim");
    need(out_size, "out_size");
    const Dims r = op->impl->output_size(dims_in(in_ndim, in_size));
    *out_ndim = (int)r.size();
    for (size_t i = 0; i < r.size(); ++i) out_size[i] = r[i];
  });
}

static pdt_status op_apply(bool adjoint, pdt_op* op, const void* src, int src_ndim, const int64_t* src_size,
                           void* dst, int dst_ndim, const int64_t* dst_size, int is_device, void* stream) {
  return guarded([&] {
    need(op, "operator");
    const Dims ds = dims_in(src_ndim, src_size), dd = dims_in(dst_ndim, dst_size);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const size_t sb = numel_of(ds) * sizeof(float2), db = numel_of(dd) * sizeof(float2);
    if (sb) need(src, "src");
    if (db) need(dst, "dst");
    if (is_device) {
      if (adjoint)
        op->impl->adjoint(static_cast<const float2*>(src), ds, static_cast<float2*>(dst), dd, st);
      else
        op->impl->forward(static_cast<const float2*>(src), ds, static_cast<float2*>(dst), dd, st);
      return;
    }
    DevBuf bs, bd;
    const float2* s = static_cast<const float2*>(dev_copy_of(src, sb, bs, st));
    bd.ensure(std::max<size_t>(db, 1));
    if (adjoint)
      op->impl->adjoint(s, ds, bd.as<float2>(), dd, st);
    else
      op->impl->forward(s, ds, bd.as<float2>(), dd, st);
    if (db) PDT_CUDA_CHECK(cudaMemcpyAsync(dst, bd.p, db, cudaMemcpyDeviceToHost, st));
    PDT_CUDA_CHECK(cudaStreamSynchronize(st));
    op->impl->check_device_errors();
  });
}

pdt_status pdt_op_forward(pdt_op* op, const void* src, int src_ndim, const int64_t* src_size, void* dst,
                          int dst_ndim, const int64_t* dst_size, int is_device, void* stream) {
  return op_apply(false, op, src, src_ndim, src_size, dst, dst_ndim, dst_size, is_device, stream);
}

pdt_status pdt_op_adjoint(pdt_op* op, const void* src, int src_ndim, const int64_t* src_size, void* dst,
                          int dst_ndim, const int64_t* dst_size, int is_device, void* stream) {
  return op_apply(true, op, src, src_ndim, src_size, dst, dst_ndim, dst_size, is_device, stream);
}

pdt_status pdt_op_describe(pdt_op* op, char* buf, size_t len) {
  return guarded([&] {
    need(op, "operator");
    need(buf, "buf");
    const std::string s = op->impl->print();
    if (len == 0) return;
    const size_t n = std::min(len - 1, s.size());
    std::memcpy(buf, s.data(), n);
    buf[n] = 0;
  });
}

pdt_status pdt_op_tuning(pdt_op* op, char* buf, size_t len) {
  return guarded([&] {
    need(op, "operator");
    need(buf, "buf");
    const std::string s = op->impl->tuning();
    if (len == 0) return;
    const size_t n = std::min(len - 1, s.size());
    std::memcpy(buf, s.data(), n);
    buf[n] = 0;
  });
}

pdt_status pdt_op_adjointness(pdt_op* op, uint64_t seed, double out[4]) {
  return guarded([&] {
    need(op, "operator");
    need(out, "out");
    OpImpl& o = *op->impl;
    const Dims isz = o.natural_input_size();
    const Dims osz2 = o.output_size(isz);
    const size_t ni = numel_of(isz), no = numel_of(osz2);
    std::mt19937_64 gen(seed);
    std::uniform_real_distribution<float> dis(0.f, 1.f);
    std::vector<float2> u(ni), p(no), Au(no), Atp(ni);
    for (auto& v : u) v = make_float2(dis(gen), dis(gen));
    for (auto& v : p) v = make_float2(dis(gen), dis(gen));
    DevBuf du, dp, dAu, dAtp;
    cudaStream_t st = 0;
    dev_copy_of(u.data(), ni * 8, du, st);
    dev_copy_of(p.data(), no * 8, dp, st);
    dAu.ensure(std::max<size_t>(no * 8, 1));
    dAtp.ensure(std::max<size_t>(ni * 8, 1));
    o.forward(du.as<float2>(), isz, dAu.as<float2>(), osz2, st);
    o.adjoint(dp.as<float2>(), osz2, dAtp.as<float2>(), isz, st);
    PDT_CUDA_CHECK(cudaMemcpy(Au.data(), dAu.p, no * 8, cudaMemcpyDeviceToHost));
    PDT_CUDA_CHECK(cudaMemcpy(Atp.data(), dAtp.p, ni * 8, cudaMemcpyDeviceToHost));
    // <a, b> = sum a * conj(b) as in iu::math::complex::dotProduct (definitions.h:66-67)
    double lr = 0, li = 0, rr = 0, ri = 0;
    for (size_t i = 0; i < no; ++i) {
      lr += (double)Au[i].x * p[i].x + (double)Au[i].y * p[i].y;
      li += (double)Au[i].y * p[i].x - (double)Au[i].x * p[i].y;
    }
    for (size_t i = 0; i < ni; ++i) {
      rr += (double)u[i].x * Atp[i].x + (double)u[i].y * Atp[i].y;
      ri += (double)u[i].y * Atp[i].x - (double)u[i].x * Atp[i].y;
    }
    out[0] = lr;
    out[1] = li;
    out[2] = rr;
    out[3] = ri;
  });
}

pdt_status pdt_opt_create(pdt_opt_kind kind, pdt_dtype dtype, pdt_opt** out) {
  return guarded([&] {
    need(out, "out");
    if (kind < PDT_OPT_TV || kind > PDT_OPT_TGV_MRI) throw Error(PDT_ERR_INVALID_ARGUMENT, "unknown optimizer kind");
    if (dtype != PDT_F32 && dtype != PDT_C64) throw Error(PDT_ERR_INVALID_ARGUMENT, "bad dtype");
    if (dtype == PDT_F32 && (kind == PDT_OPT_TV_OP || kind == PDT_OPT_TGV_OP || kind == PDT_OPT_TGV_MRI))
      throw Error(PDT_ERR_UNSUPPORTED, "optimizers with an MRI operator are complex (PDT_C64)");
    auto h = std::make_unique<pdt_opt>();
    h->impl = std::make_unique<OptImpl>(kind, dtype);
    *out = h.release();
  });
}

pdt_status pdt_opt_destroy(pdt_opt* opt) {
  return guarded([&] { delete opt; });
}

pdt_status pdt_opt_get_params(pdt_opt* opt, pdt_params* out) {
  return guarded([&] {
    need(opt, "optimizer");
    *need(out, "out") = opt->impl->params_;
  });
}

pdt_status pdt_opt_set_params(pdt_opt* opt, const pdt_params* params) {
  return guarded([&] {
    need(opt, "optimizer");
    opt->impl->params_ = *need(params, "params");
  });
}

pdt_status pdt_opt_set_operator(pdt_opt* opt, pdt_op* op) {
  return guarded([&] {
    need(opt, "optimizer");
    need(op, "operator");
    opt->impl->set_operator(op->impl);
  });
}

pdt_status pdt_opt_set_noisy_data(pdt_opt* opt, const void* f, int ndim, const int64_t* size, int is_device,
                                  void* stream) {
  return guarded([&] {
    need(opt, "optimizer");
    const Dims d = dims_in(ndim, size);
    if (numel_of(d)) need(f, "data");
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : opt->impl->own_stream();
    opt->impl->set_noisy_data(f, d, is_device != 0, st);
    if (!stream) PDT_CUDA_CHECK(cudaStreamSynchronize(st));
  });
}

pdt_status pdt_opt_set_input0(pdt_opt* opt, const void* u0, int ndim, const int64_t* size, int is_device,
                              void* stream) {
  return guarded([&] {
    need(opt, "optimizer");
    const Dims d = dims_in(ndim, size);
    if (numel_of(d)) need(u0, "input");
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : opt->impl->own_stream();
    opt->impl->set_input0(u0, d, is_device != 0, st);
    if (!stream) PDT_CUDA_CHECK(cudaStreamSynchronize(st));
  });
}

pdt_status pdt_opt_solve(pdt_opt* opt, int verbose, void* stream) {
  return guarded([&] {
    need(opt, "optimizer");
    opt->impl->check_ready();
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : opt->impl->own_stream();
    opt->impl->solve(verbose != 0, st);
    if (!stream) {
      PDT_CUDA_CHECK(cudaStreamSynchronize(st));
      opt->impl->check_device(st);
    }
  });
}

pdt_status pdt_opt_set_steps(pdt_opt* opt, double tau, double sigma) {
  return guarded([&] {
    need(opt, "optimizer");
    if (!(tau >= 0) || !(sigma >= 0)) throw Error(PDT_ERR_INVALID_ARGUMENT, "step sizes must be >= 0");
    opt->impl->step_tau_ = (float)tau;
    opt->impl->step_sigma_ = (float)sigma;
  });
}

pdt_status pdt_debug_drop_arrival(int on) {
  return guarded([&] {
    cartesian_set_drop_arrival(on);
    cnn_set_drop_arrival(on);
  });
}

pdt_status pdt_opt_status(pdt_opt* opt, void* stream) {
  return guarded([&] {
    need(opt, "optimizer");
    opt->impl->check_device(stream ? static_cast<cudaStream_t>(stream) : opt->impl->own_stream());
  });
}

pdt_status pdt_opt_result_size(pdt_opt* opt, int* ndim, int64_t* size) {
  return guarded([&] {
    need(opt, "optimizer");
    need(ndim, "ndim");
    need(size, "size");
    const Dims d = opt->impl->result_size();
    *ndim = (int)d.size();
    for (size_t i = 0; i < d.size(); ++i) size[i] = d[i];
  });
}

pdt_status pdt_opt_get_result(pdt_opt* opt, void* dst, int is_device, void* stream) {
  return guarded([&] {
    need(opt, "optimizer");
    need(dst, "dst");
    opt->impl->result_size();  // "There is no result yet!" before touching the device
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : opt->impl->own_stream();
    opt->impl->get_result(dst, is_device != 0, st);
    if (!stream) PDT_CUDA_CHECK(cudaStreamSynchronize(st));
  });
}

pdt_status pdt_opt_set_input0_uv(pdt_opt* opt, const void* u0, const void* v0, int ndim, const int64_t* size,
                                 int is_device, void* stream) {
  return guarded([&] {
    need(opt, "optimizer");
    const Dims d = dims_in(ndim, size);
    if (numel_of(d)) need(u0, "input");
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : opt->impl->own_stream();
    opt->impl->set_input0_uv(u0, v0, d, is_device != 0, st);
    if (!stream) PDT_CUDA_CHECK(cudaStreamSynchronize(st));
  });
}

pdt_status pdt_opt_get_field(pdt_opt* opt, int field, void* dst, int is_device, void* stream) {
  return guarded([&] {
    need(opt, "optimizer");
    need(dst, "dst");
    opt->impl->result_size();
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : opt->impl->own_stream();
    opt->impl->get_field(field, dst, is_device != 0, st);
    if (!stream) PDT_CUDA_CHECK(cudaStreamSynchronize(st));
  });
}

pdt_status pdt_opt_set_field(pdt_opt* opt, int field, const void* src, int is_device, void* stream) {
  return guarded([&] {
    need(opt, "optimizer");
    need(src, "source");
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : opt->impl->own_stream();
    opt->impl->set_field(field, src, is_device != 0, st);
    if (!stream) PDT_CUDA_CHECK(cudaStreamSynchronize(st));
  });
}

pdt_status pdt_opt_gap(pdt_opt* opt, void* stream, double out[6]) {
  return guarded([&] {
    need(opt, "optimizer");
    need(out, "out");
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : opt->impl->own_stream();
    opt->impl->gap(st, out);
  });
}

pdt_status pdt_opt_energy(pdt_opt* opt, void* stream, double out[4]) {
  return guarded([&] {
    need(opt, "optimizer");
    need(out, "out");
    opt->impl->check_ready();
    opt->impl->result_size();
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : opt->impl->own_stream();
    opt->impl->energy(st, out);
  });
}

pdt_status pdt_op_norm(pdt_op* op, int iters, uint64_t seed, double* out) {
  return guarded([&] {
    need(op, "operator");
    need(out, "out");
    if (iters < 1) throw Error(PDT_ERR_INVALID_ARGUMENT, "iters must be >= 1");
    OpImpl& o = *op->impl;
    const Dims isz = o.natural_input_size();
    const Dims osz = o.output_size(isz);
    const size_t ni = numel_of(isz), no = numel_of(osz);
    std::mt19937_64 gen(seed);
    std::normal_distribution<float> dis(0.f, 1.f);
    std::vector<float2> x0(ni);
    for (auto& v : x0) v = make_float2(dis(gen), dis(gen));
    DevBuf x, y;
    cudaStream_t st = 0;
    dev_copy_of(x0.data(), ni * 8, x, st);
    y.ensure(std::max<size_t>(no * 8, 1));
    double lam = 0;
    double nx = std::sqrt(reduce_dist2(true, x.p, nullptr, ni, st));
    for (int k = 0; k < iters; ++k) {
      launch_scale(x.as<float2>(), (float)(1.0 / nx), ni, st);  // |x| = 1
      o.forward(x.as<float2>(), isz, y.as<float2>(), osz, st);
      o.adjoint(y.as<float2>(), osz, x.as<float2>(), isz, st);  // x <- K^H K x
      nx = std::sqrt(reduce_dist2(true, x.p, nullptr, ni, st));
      lam = nx;  // Rayleigh growth of a unit vector
    }
    *out = std::sqrt(lam);
  });
}

pdt_status pdt_dist2(pdt_dtype dtype, const void* a, const void* b, size_t n, void* stream, double* out) {
  return guarded([&] {
    need(a, "a");
    need(out, "out");
    *out = reduce_dist2(dtype == PDT_C64, a, b, n, static_cast<cudaStream_t>(stream));
  });
}

pdt_status pdt_batch_create(pdt_batch** out) {
  return guarded([&] {
    need(out, "out");
    auto h = std::make_unique<pdt_batch>();
    h->impl = std::make_unique<BatchImpl>();
    *out = h.release();
  });
}

pdt_status pdt_batch_destroy(pdt_batch* b) {
  return guarded([&] { delete b; });
}

pdt_status pdt_batch_add(pdt_batch* b, pdt_opt* opt) {
  return guarded([&] {
    need(b, "batch");
    need(opt, "optimizer");
    b->impl->add(opt->impl.get());
  });
}

pdt_status pdt_batch_solve(pdt_batch* b, int verbose, void* stream) {
  return guarded([&] {
    need(b, "batch");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    b->impl->solve(verbose != 0, st);
    if (!stream) {
      PDT_CUDA_CHECK(cudaStreamSynchronize(st));
      b->impl->check_device(st);
    }
  });
}

pdt_status pdt_opt_profile(pdt_opt* opt, int iters, void* stream, int max_phases, int* nphases, char* names,
                           size_t names_len, double* ms) {
  return guarded([&] {
    need(opt, "optimizer");
    need(nphases, "nphases");
    if (iters < 1) throw Error(PDT_ERR_INVALID_ARGUMENT, "iters must be >= 1");
    opt->impl->check_ready();
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : opt->impl->own_stream();
    std::vector<std::string> nm;
    std::vector<double> t;
    opt->impl->profile(iters, st, nm, t);
    *nphases = (int)nm.size();
    std::string joined;
    for (size_t i = 0; i < nm.size(); ++i) {
      if (i < (size_t)max_phases && ms) ms[i] = t[i];
      joined += (i ? "," : "") + nm[i];
    }
    if (names && names_len) {
      const size_t n = std::min(names_len - 1, joined.size());
      std::memcpy(names, joined.data(), n);
      names[n] = 0;
    }
  });
}

}  // extern "C"
