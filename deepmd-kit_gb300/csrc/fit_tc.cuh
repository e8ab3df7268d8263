// Tensor-core fitting-net GEMM with fused epilogues (mixed-precision form).
#pragma once

#include <cuda_bf16.h>

#include "common.cuh"

namespace dpgb {

enum FitMode { kFitFwd = 0, kFitFwdLast = 1, kFitBwd = 2, kFitStore = 3 };

// One GEMM  acc[M, N] = A[M, K] . B^T  (A bf16 row-major with leading
// dimension lda, B bf16 [N, K] row-major) and its epilogue:
//  kFitFwd:     t = tanh(acc + bias); y = t*idt (+ Xs); Yf, Yb (bf16), Tt = t
//  kFitFwdLast: as kFitFwd, then e = y . w_out + b_out, dPb = w_out*idt*(1-t^2)
//  kFitBwd:     dx = acc (+ dYup); dXf = dx; dPb = dx*idt_lo*(1 - T_lo^2)
//  kFitStore:   out = acc
struct FitGemm {
  int mode;
  int M, N, K, lda;
  const __nv_bfloat16* A;
  const __nv_bfloat16* B;
  const float* bias;
  const float* idt;
  const float* Xs;
  int ldxs, skip;
  float* Yf;
  __nv_bfloat16* Yb;
  float* Tt;
  int ldy;
  const float* w_out;
  float b_out;
  double* e_out;
  __nv_bfloat16* dPb;
  const float* dYup;
  int lddyup;
  float* dXf;
  const float* idt_lo;
  const float* T_lo;
  float* out;
  int ldo;
};

int fit_tc_eligible(const dpgb_se_a_desc& d);
int launch_fit_gemm(const FitGemm& g, int* err, cudaStream_t st);

}  // namespace dpgb
