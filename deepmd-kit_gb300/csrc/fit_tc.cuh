// Tensor-core fitting-net GEMM with fused epilogues (mixed-precision form).
#pragma once

#include <cuda_bf16.h>

#include "common.cuh"

namespace dpgb {

enum FitMode { kFitFwd = 0, kFitFwdLast = 1, kFitBwd = 2, kFitStore = 3 };

// One GEMM over the type-sorted rows of all atom types (type t owns sorted
// rows [row0[t], row0[t+1]) and uses its own weights):
//   acc[m, n] = A_hi[m, :] . B_hi[n, :] + A_lo[m, :] . B_hi[n, :] + A_hi[m, :] . B_lo[n, :]
// in split BF16: hi is an operand's BF16 rounding, lo the BF16 rounding of
// the remainder, so hi + lo carries ~16 significant bits.  The A_lo term is
// there when A_lo is set; the weight's high part sits in columns [0, K) of
// the B image and its low part in columns [Kp, Kp + K) (Kp = K rounded up to
// 64, zeros between).  (A bf16 [rows, lda], B image bf16 [type][N][2 Kp].)
// The epilogue:
//  kFitFwd:     t = tanh(acc + bias_t); y = t*idt_t (+ Xs); Yf, Yb (bf16 hi),
//               Yb_lo (bf16 lo, when set), Tt = t
//  kFitFwdLast: as kFitFwd, then e = y . w_out_t + b_out[t],
//               dPb = w_out_t * idt_t * (1 - t^2)        (needs N <= 256)
//  kFitBwd:     dx = acc (+ dYup); dXf = dx; dPb = dx * idt_lo_t * (1 - T_lo^2)
//  (dPb_lo, when set, receives the low part of dPb)
//  kFitStore:   out = acc
// Per-type parameter arrays are laid out [type][N].
struct FitGemm {
  int mode;
  int N, K, lda;
  int Kp;                    // K rounded up to 64 (the B image holds 2 Kp columns)
  const __nv_bfloat16* A_lo;  // low part of A, same layout, or null
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
  __nv_bfloat16* Yb_lo;
  float* Tt;
  int ldy;
  const float* w_out;  // [type][N]
  float b_out[8];
  double* e_out;
  __nv_bfloat16* dPb;
  __nv_bfloat16* dPb_lo;
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
// The product runs in three split-BF16 segments (dP1 hi . W1 hi + dP1 lo .
// W1 hi + dP1 hi . W1 lo).
struct FitDxyz {
  int ntypes;
  int row0[9], tile0[9];   // as FitGemm
  int K, Kp;               // width of the first hidden layer; K rounded up to 64
  int ng, nnei;
  const __nv_bfloat16* A;  // dP1 high part [rows, lda] (type-sorted rows)
  const __nv_bfloat16* A_lo;  // dP1 low part, same layout
  int lda;
  const __nv_bfloat16* B;  // W1 per type [type][16 ng][2 Kp] (high part, then low part)
  const float* xyz;        // [rows (original order)][4][ng]
  const int* sorted_rows;  // sorted row -> original row
  float* dxyz;             // [rows (original order)][ng][4]
};

int fit_tc_eligible(const dpgb_se_a_desc& d);
int launch_fit_gemm(const FitGemm& g, int* err, cudaStream_t st);
int launch_fit_dxyz(const FitDxyz& f, int* err, cudaStream_t st);

}  // namespace dpgb
