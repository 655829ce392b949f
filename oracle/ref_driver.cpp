// ref_driver.cpp -- C entry points into the reference's own optimizers and Cartesian operators, compiled for
// the CPU by oracle/ref_build.py (with the host stand-in for ImageUtilities in oracle/ref_shim/).
//
// TEST INFRASTRUCTURE ONLY: tests use oracle/_ref/libpdtref.so to pin the oracle restatement and to write
// golden vectors; nothing of the product loads it.
//
// Each entry point does what the reference's Python bindings do (python/pyMriReconstruction.cpp:67-110,
// python/pyDenoising.cpp:50-93): wrap the caller's arrays in ImageUtilities memory (numpy (C, H, W) in C
// order = ImageUtilities (W, H, C)), add the constants in their positional order, set the parameters,
// solve, and copy getResult() out. The reference's console output is discarded. Returns 0, or 1 with the
// exception's text in ref_last_error().
#include <cstring>
#include <iostream>
#include <memory>
#include <sstream>
#include <string>

#include "operator/mricartesianoperator.h"
#include "optimizer/tgvmrioptimizer.h"
#include "optimizer/tgvoptimizer.h"
#include "optimizer/tgvoptimizerwithop.h"
#include "optimizer/tvoptimizer.h"
#include "optimizer/tvoptimizerwithop.h"

namespace {

typedef iu::LinearDeviceMemory<float2, 2> Img;
typedef iu::LinearDeviceMemory<float2, 3> Ksp;

std::string g_err;

struct Quiet {  // the reference prints its parameters and progress on every solve
  std::ostringstream sink;
  std::streambuf* old;
  Quiet() : old(std::cout.rdbuf(sink.rdbuf())) {}
  ~Quiet() { std::cout.rdbuf(old); }
};

template <class F>
int guarded(F&& f) {
  try {
    Quiet q;
    f();
    return 0;
  } catch (const std::exception& e) {
    g_err = e.what();
    return 1;
  }
}

template <class Op>
std::shared_ptr<OperatorBase<Img, Ksp>> cart_op(int W, int Hf, int C, const float2* sens, const float* mask) {
  auto op = std::make_shared<Op>();
  iu::LinearHostMemory<float2, 3> s(const_cast<float2*>(sens), iu::Size<3>({(unsigned)W, (unsigned)Hf, (unsigned)C}),
                                    true);
  iu::LinearHostMemory<float, 2> m(const_cast<float*>(mask), iu::Size<2>({(unsigned)W, (unsigned)Hf}), true);
  op->addConstant(s);
  op->addConstant(m);
  return op;
}

std::shared_ptr<OperatorBase<Img, Ksp>> make_op(int roos, int W, int Hf, int C, const float2* sens, const float* mask) {
  if (roos) return cart_op<MriCartesianRemoveROOSOperator<Img, Ksp>>(W, Hf, C, sens, mask);
  return cart_op<MriCartesianOperator<Img, Ksp>>(W, Hf, C, sens, mask);
}

std::shared_ptr<Ksp> kdata(int W, int Hf, int C, const float2* f) {
  return std::make_shared<Ksp>(const_cast<float2*>(f), iu::Size<3>({(unsigned)W, (unsigned)Hf, (unsigned)C}), false);
}

template <class Opt>
void copy_result(Opt& opt, void* out, size_t bytes) {
  std::memcpy(out, opt.getResult()->data(), bytes);
}

// TvOptimizer (tvoptimizer.cu:76-125) and TgvOptimizer (tgvoptimizer.cu:80-141) on a float (cplx = 0)
// or float2 (cplx = 1) W x H image.
template <class T>
void denoise(int tgv, int W, int H, const void* f, float lambda, float alpha0, float alpha1, unsigned max_iter,
                    void* out) {
  typedef iu::LinearDeviceMemory<T, 2> M;
  auto fd = std::make_shared<M>(static_cast<T*>(const_cast<void*>(f)), iu::Size<2>({(unsigned)W, (unsigned)H}), false);
  if (tgv) {
    TgvOptimizer<M, M> opt;
    opt.setNoisyData(fd);
    auto& p = opt.getParameters();
    p.lambda = lambda;
    p.alpha0 = alpha0;
    p.alpha1 = alpha1;
    p.max_iter = max_iter;
    p.check = 1u << 30;
    opt.solve(false);
    copy_result(opt, out, sizeof(T) * (size_t)W * H);
  } else {
    TvOptimizer<M, M> opt;
    opt.setNoisyData(fd);
    auto& p = opt.getParameters();
    p.lambda = lambda;
    p.max_iter = max_iter;
    p.check = 1u << 30;
    opt.solve(false);
    copy_result(opt, out, sizeof(T) * (size_t)W * H);
  }
}

}  // namespace

extern "C" {

const char* ref_last_error() { return g_err.c_str(); }

// MriCartesianOperator / MriCartesianRemoveROOSOperator executeForward (adjoint = 0) or executeAdjoint
// (mricartesianoperator.cu:196-265, 320-414) through OperatorBase::forward / adjoint.
int ref_cart_apply(int roos, int adjoint, int W, int Hf, int C, const float2* sens, const float* mask, const float2* src,
                   float2* dst) {
  return guarded([&] {
    auto op = make_op(roos, W, Hf, C, sens, mask);
    const unsigned Hi = roos ? Hf / 2 : Hf;
    Img u(iu::Size<2>({(unsigned)W, Hi}));
    Ksp k(iu::Size<3>({(unsigned)W, (unsigned)Hf, (unsigned)C}));
    if (adjoint) {
      std::memcpy(k.data(), src, k.bytes());
      op->adjoint(k, u);
      std::memcpy(dst, u.data(), u.bytes());
    } else {
      std::memcpy(u.data(), src, u.bytes());
      op->forward(u, k);
      std::memcpy(dst, k.data(), k.bytes());
    }
  });
}

// TgvMriOptimizer<float2 image, float2 k-space> (tgvmrioptimizer.cu:93-203); u0 = NULL starts from A^H f.
int ref_tgv_mri(int roos, int W, int Hf, int C, const float2* sens, const float* mask, const float2* f, const float2* u0,
                float alpha0, float alpha1, float reduction, unsigned max_iter, float2* u_out) {
  return guarded([&] {
    TgvMriOptimizer<Img, Ksp> opt;
    opt.setOperator(make_op(roos, W, Hf, C, sens, mask));
    opt.setNoisyData(kdata(W, Hf, C, f));
    const unsigned Hi = roos ? Hf / 2 : Hf;
    if (u0) opt.setInput0(Img(const_cast<float2*>(u0), iu::Size<2>({(unsigned)W, Hi}), true));
    auto& p = opt.getParameters();
    p.alpha0 = alpha0;
    p.alpha1 = alpha1;
    p.reduction = reduction;
    p.max_iter = max_iter;
    p.check = 1u << 30;
    opt.solve(false);
    copy_result(opt, u_out, sizeof(float2) * (size_t)W * Hi);
  });
}

// TgvOptimizerWithOp (variant 0, tgvoptimizerwithop.cu:89-179) or TvOptimizerWithOp (variant 1,
// tvoptimizerwithop.cu:86-164) with a Cartesian operator.
int ref_with_op(int variant, int roos, int W, int Hf, int C, const float2* sens, const float* mask, const float2* f,
                float lambda, float alpha0, float alpha1, unsigned max_iter, float2* u_out) {
  return guarded([&] {
    const unsigned Hi = roos ? Hf / 2 : Hf;
    if (variant == 0) {
      TgvOptimizerWithOp<Img, Ksp> opt;
      opt.setOperator(make_op(roos, W, Hf, C, sens, mask));
      opt.setNoisyData(kdata(W, Hf, C, f));
      auto& p = opt.getParameters();
      p.lambda = lambda;
      p.alpha0 = alpha0;
      p.alpha1 = alpha1;
      p.max_iter = max_iter;
      p.check = 1u << 30;
      opt.solve(false);
      copy_result(opt, u_out, sizeof(float2) * (size_t)W * Hi);
    } else {
      TvOptimizerWithOp<Img, Ksp> opt;
      opt.setOperator(make_op(roos, W, Hf, C, sens, mask));
      opt.setNoisyData(kdata(W, Hf, C, f));
      auto& p = opt.getParameters();
      p.lambda = lambda;
      p.max_iter = max_iter;
      p.check = 1u << 30;
      opt.solve(false);
      copy_result(opt, u_out, sizeof(float2) * (size_t)W * Hi);
    }
  });
}

int ref_denoise(int tgv, int cplx, int W, int H, const void* f, float lambda, float alpha0, float alpha1,
                unsigned max_iter, void* out) {
  return guarded([&] {
    if (cplx)
      denoise<float2>(tgv, W, H, f, lambda, alpha0, alpha1, max_iter, out);
    else
      denoise<float>(tgv, W, H, f, lambda, alpha0, alpha1, max_iter, out);
  });
}

}  // extern "C"
