// Tensor-core fitting-net GEMM with fused epilogues (mixed-precision form).
#pragma once

#include <cuda_bf16.h>

#include "common.cuh"

namespace dpgb {

enum FitMode { kFitFwd = 0, kFitFwdLast = 1, kFitBwd = 2, kFitStore = 3 };

// One GEMM over the type-sorted rows of all atom types (type t owns sorted
// rows [row0[t], row0[t+1]) and uses its own weights):
//   acc[m, n] = A[m, :] . B_t[n, :]      (A bf16 [rows, lda], B_t bf16 [N, K])
// and its epilogue:
//  kFitFwd:     t = tanh(acc + bias_t); y = t*idt_t (+ Xs); Yf, Yb (bf16), Tt = t
//  kFitFwdLast: as kFitFwd, then e = y . w_out_t + b_out[t],
//               dPb = w_out_t * idt_t * (1 - t^2)        (needs N <= 256)
//  kFitBwd:     dx = acc (+ dYup); dXf = dx; dPb = dx * idt_lo_t * (1 - T_lo^2)
//  kFitStore:   out = acc
// Per-type parameter arrays are laid out [type][N] (B: [type][N][K]).
struct FitGemm {
  int mode;
  int N, K, lda;
  int ntypes;
  int row0[9];   // sorted-row offsets of the types
  int tile0[9];  // prefix of 128-row tiles per type
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
  const float* w_out;  // [type][N]
  float b_out[8];
  double* e_out;
  __nv_bfloat16* dPb;
  const float* dYup;   // [rows][lddyup], or w_out-like [type][N] when lddyup == 0
  int lddyup;
  float* dXf;
  const float* idt_lo;
  const float* T_lo;
  float* out;
  int ldo;
};

// dE/dD of the first fitting layer (dD = dP1 . W1 per type) folded straight
// into dE/dxyz, dD never stored: for row r, dxyz[r][n][c] = (sum_m dD[n][m]
// xyz[c][m] + [n < 16] sum_n' dD[n'][n] xyz[c][n']) / nnei, with dD[n][m] =
// column 16 n + m (axis width 16).
struct FitDxyz {
  int ntypes;
  int row0[9], tile0[9];   // as FitGemm
  int K;                   // width of the first hidden layer
  int ng, nnei;
  const __nv_bfloat16* A;  // dP1 [rows, lda] (type-sorted rows)
  int lda;
  const __nv_bfloat16* B;  // W1 per type [type][16 ng][K]
  const float* xyz;        // [rows (original order)][4][ng]
  const int* sorted_rows;  // sorted row -> original row
  float* dxyz;             // [rows (original order)][ng][4]
};

int fit_tc_eligible(const dpgb_se_a_desc& d);
int launch_fit_gemm(const FitGemm& g, int* err, cudaStream_t st);
int launch_fit_dxyz(const FitDxyz& f, int* err, cudaStream_t st);

}  // namespace dpgb
