// Tensor-core (tcgen05) energy fitting net for the mixed-precision DeepPot:
// forward tanh layers, the output layer and the input-gradient backward
// (dE/dD) as BF16 GEMMs with FP32 TMEM accumulators and fused epilogues
// (deepmd/pt/model/task/fitting.py:734-899 semantics; hidden layer
// y = tanh(x W + b) * idt (+ x when the widths match)).
//
// One launch covers the rows of every atom type (each 128-row tile belongs to
// one type and uses that type's weights).  A CTA computes a 128 x BN tile; K is
// streamed in chunks of 64 through an S-stage ring filled by TMA (one 2D
// tensor copy per operand and stage, 128-byte swizzled rows, completion
// counted in bytes on the stage's "full" barrier) by one producer thread,
// while one MMA thread consumes the stages and releases each through its
// "empty" barrier when the MMAs reading it commit.  Rows past the operand's
// end and K past its width arrive as zeros.  The epilogue runs one thread
// per row in each of WG warp groups, which split the tile's columns; each
// thread stores 16 consecutive columns at a time (64-byte segments).
#include <cuda.h>
#include <cudaTypedefs.h>

#include "fit_tc.cuh"
#include "tc.cuh"

namespace dpgb {
namespace {

constexpr int kKC = 64;

// tanh to a few units in the last place (the hardware tanh.approx.f32 is
// good to about 2^-11 relative, which alone moved forces by ~4e-4 of their
// RMS): below 1/16 the odd series x - x^3/3 + 2x^5/15 - 17x^7/315 (next
// term 62/2835 x^9 < 4e-13 there); above, 1 - 2 / (e^{2|x|} + 1) with the
// exponential and the division of CUDA's fast intrinsics (relative error of
// a few 1e-7 before the subtraction, which only shrinks it).
__device__ __forceinline__ float tanh_acc(float x) {
  const float a = fabsf(x);
  if (a < 0.0625f) {
    const float x2 = x * x;
    return x * fmaf(x2, fmaf(x2, fmaf(x2, -17.f / 315.f, 2.f / 15.f), -1.f / 3.f), 1.f);
  }
  const float e = __expf(2.f * fminf(a, 12.f));
  return copysignf(1.f - __fdividef(2.f, e + 1.f), x);
}

// high and low BF16 parts of an FP32 value (hi + lo carries ~16 bits)
__device__ __forceinline__ void split_bf16(float v, __nv_bfloat16& hi, __nv_bfloat16& lo) {
  hi = __float2bfloat16_rn(v);
  lo = __float2bfloat16_rn(v - __bfloat162float(hi));
}


__device__ __forceinline__ void ld16f(const float* p, float* v) {
  const float4* q = reinterpret_cast<const float4*>(p);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const float4 x = q[i];
    v[4 * i] = x.x;
    v[4 * i + 1] = x.y;
    v[4 * i + 2] = x.z;
    v[4 * i + 3] = x.w;
  }
}
__device__ __forceinline__ void st16f(float* p, const float* v) {
  float4* q = reinterpret_cast<float4*>(p);
#pragma unroll
  for (int i = 0; i < 4; ++i) q[i] = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
}
__device__ __forceinline__ void st16b(__nv_bfloat16* p, const float* v) {
  __nv_bfloat162 h[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) h[i] = __floats2bfloat162_rn(v[2 * i], v[2 * i + 1]);
  uint4* q = reinterpret_cast<uint4*>(p);
  q[0] = *reinterpret_cast<uint4*>(&h[0]);
  q[1] = *reinterpret_cast<uint4*>(&h[4]);
}
// 16 values as BF16 high parts at p and, when lo is set, low parts at lo
__device__ __forceinline__ void st16b_split(__nv_bfloat16* p, __nv_bfloat16* lo, const float* v) {
  if (!lo) {
    st16b(p, v);
    return;
  }
  __nv_bfloat16 h[16], l[16];
#pragma unroll
  for (int i = 0; i < 16; ++i) split_bf16(v[i], h[i], l[i]);
  uint4* q = reinterpret_cast<uint4*>(p);
  q[0] = *reinterpret_cast<uint4*>(&h[0]);
  q[1] = *reinterpret_cast<uint4*>(&h[8]);
  uint4* ql = reinterpret_cast<uint4*>(lo);
  ql[0] = *reinterpret_cast<uint4*>(&l[0]);
  ql[1] = *reinterpret_cast<uint4*>(&l[8]);
}

// NA: parts of A (1: hi, 2: hi and lo); the weight always comes as hi and
// lo.  A stage holds one K chunk of every part, so each part is read once.
template <int BN, int S, int WG, int NA>
__global__ void __launch_bounds__(128 * WG)
fit_gemm_kernel(const __grid_constant__ CUtensorMap tma_a, const __grid_constant__ CUtensorMap tma_alo,
                const __grid_constant__ CUtensorMap tma_b, FitGemm g, int* __restrict__ err) {
  extern __shared__ unsigned char smem_raw[];
  // swizzled TMA tiles want 1024-byte aligned stages
  unsigned char* smem = smem_raw + ((1024 - (tc::smem_u32(smem_raw) & 1023)) & 1023);
  __shared__ uint64_t full[S], empty[S], done;
  __shared__ uint32_t s_tmem;
  __shared__ float s_e[2 * (WG - 1) * 128 + 2];  // compensated partial energies of column groups 1 .. WG-1
  constexpr int SA = 128 * kKC * 2, SB = BN * kKC * 2, STAGE = NA * SA + 2 * SB;
  constexpr uint32_t kTmemCols = BN <= 32 ? 32 : (BN <= 64 ? 64 : (BN <= 128 ? 128 : 256));
  static_assert(BN % 16 == 0 && BN <= 256 && SB % 1024 == 0, "whole 16-column loads, 1024-byte aligned stages");
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  int t = 0;
  while (t + 1 < g.ntypes && g.tile0[t + 1] <= (int)blockIdx.y) ++t;
  const int m0 = g.row0[t] + ((int)blockIdx.y - g.tile0[t]) * 128;
  const int rows_valid = min(128, g.row0[t + 1] - m0);
  const int n0 = blockIdx.x * BN;
  const int nt = min(BN, g.N - n0);  // multiple of 16
  if (warp == 0) tc::tmem_alloc(&s_tmem, kTmemCols);
  if (tid == 0) {
    for (int s = 0; s < S; ++s) {
      tc::mbar_init(&full[s], 1);
      tc::mbar_init(&empty[s], 1);
    }
    tc::mbar_init(&done, 1);
    tc::fence_mbar_init();
  }
  __syncthreads();
  tc::fence_after();
  const uint32_t tbase = s_tmem;
  // stage layout: A hi [, A lo], B hi, B lo
  const int nchunk = (g.K + kKC - 1) / kKC;
  bool ok = true;
  if (warp == 1 && lane == 0) {
    // producer: chunk i into stage i % S once the MMAs of chunk i - S released it
    for (int i = 0; i < nchunk && ok; ++i) {
      const int s = i % S;
      if (i >= S) ok = tc::mbar_wait(&empty[s], ((i / S) - 1) & 1, err);
      if (!ok) break;
      const uint32_t a0 = tc::smem_u32(smem + s * STAGE), b0 = a0 + NA * SA;
      tc::mbar_expect_tx(&full[s], STAGE);
      tc::tma_load_2d(a0, &tma_a, i * kKC, m0, &full[s]);
      if (NA == 2) tc::tma_load_2d(a0 + SA, &tma_alo, i * kKC, m0, &full[s]);
      tc::tma_load_2d(b0, &tma_b, i * kKC, t * g.N + n0, &full[s]);
      tc::tma_load_2d(b0 + SB, &tma_b, g.Kp + i * kKC, t * g.N + n0, &full[s]);
    }
  } else if (warp == 0 && lane == 0) {
    // MMA issuer: 4 steps of K = 16 per chunk (zeros past K add nothing),
    // each hi.hi (+ lo.hi) + hi.lo
    const uint32_t idesc = tc::idesc_bf16_f32(128, nt);
    for (int i = 0; i < nchunk && ok; ++i) {
      const int s = i % S;
      ok = tc::mbar_wait(&full[s], (i / S) & 1, err);
      if (!ok) break;
      tc::fence_after();
      const uint32_t a0 = tc::smem_u32(smem + s * STAGE), b0 = a0 + NA * SA;
#pragma unroll
      for (int ks = 0; ks < kKC / 16; ++ks) {
        tc::mma_bf16(tbase, tc::smem_desc_sw128(a0 + ks * 32), tc::smem_desc_sw128(b0 + ks * 32), idesc,
                     (i > 0 || ks > 0) ? 1u : 0u);
        if (NA == 2)
          tc::mma_bf16(tbase, tc::smem_desc_sw128(a0 + SA + ks * 32), tc::smem_desc_sw128(b0 + ks * 32), idesc, 1u);
        tc::mma_bf16(tbase, tc::smem_desc_sw128(a0 + ks * 32), tc::smem_desc_sw128(b0 + SB + ks * 32), idesc, 1u);
      }
      tc::mma_commit(&empty[s]);
    }
    tc::mma_commit(&done);
  }
  __syncwarp();
  ok = tc::mbar_wait(&done, 0, err) && ok;
  tc::fence_after();
  ok = __syncthreads_and(ok) != 0;
  // epilogue: thread = row (warp quadrant q = TMEM lanes 32 q ..), the
  // WG warp groups take the tile's 16-column groups in turn
  const int q = warp & 3, h = warp >> 2;
  const int r = q * 32 + lane;
  const int m = m0 + r;
  const bool valid = r < rows_valid;
  float e_hi = 0.f, e_lo = 0.f;  // output layer: compensated sum of y w over this group's columns
  if (ok) {
    const float* bias = g.bias ? g.bias + (size_t)t * g.N : nullptr;
    const float* idt = g.idt ? g.idt + (size_t)t * g.N : nullptr;
    const float* idt_lo = g.idt_lo ? g.idt_lo + (size_t)t * g.N : nullptr;
    const float* wo = g.w_out ? g.w_out + (size_t)t * g.N : nullptr;
    for (int c0 = h * 16; c0 < nt; c0 += 16 * WG) {
      float v[16];
      tc::tmem_ld16(tc::taddr(tbase, q * 32, c0), v);
      tc::tmem_ld_wait();
      if (!valid) continue;
      const int n = n0 + c0;
      if (g.mode == kFitFwd || g.mode == kFitFwdLast) {
        float bb[16], id[16], xs[16], y[16], tv[16];
        ld16f(bias + n, bb);
        if (idt) ld16f(idt + n, id);
        if (g.skip) ld16f(g.Xs + (size_t)m * g.ldxs + n, xs);
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          tv[i] = tanh_acc(v[i] + bb[i]);
          y[i] = idt ? tv[i] * id[i] : tv[i];
          if (g.skip) y[i] += xs[i];
        }
        if (g.mode == kFitFwd) {
          st16f(g.Yf + (size_t)m * g.ldy + n, y);
          st16f(g.Tt + (size_t)m * g.ldy + n, tv);
          st16b_split(g.Yb + (size_t)m * g.ldy + n, g.Yb_lo ? g.Yb_lo + (size_t)m * g.ldy + n : nullptr, y);
        } else {
          float w[16], dp[16];
          ld16f(wo + n, w);
#pragma unroll
          for (int i = 0; i < 16; ++i) {
            const float pr = y[i] * w[i];
            comp_add(e_hi, e_lo, pr);
            e_lo += fmaf(y[i], w[i], -pr);  // the product's rounding error
            dp[i] = w[i] * (idt ? id[i] : 1.f) * (1.f - tv[i] * tv[i]);
          }
          st16b_split(g.dPb + (size_t)m * g.ldy + n, g.dPb_lo ? g.dPb_lo + (size_t)m * g.ldy + n : nullptr, dp);
        }
      } else if (g.mode == kFitBwd) {
        float dx[16], up[16], tl[16], il[16], dp[16];
#pragma unroll
        for (int i = 0; i < 16; ++i) dx[i] = v[i];
        if (g.dYup) {
          ld16f(g.lddyup ? g.dYup + (size_t)m * g.lddyup + n : g.dYup + (size_t)t * g.N + n, up);
#pragma unroll
          for (int i = 0; i < 16; ++i) dx[i] += up[i];
        }
        if (g.dXf) st16f(g.dXf + (size_t)m * g.ldy + n, dx);
        ld16f(g.T_lo + (size_t)m * g.ldy + n, tl);
        if (idt_lo) ld16f(idt_lo + n, il);
#pragma unroll
        for (int i = 0; i < 16; ++i) dp[i] = dx[i] * (idt_lo ? il[i] : 1.f) * (1.f - tl[i] * tl[i]);
        st16b_split(g.dPb + (size_t)m * g.ldy + n, g.dPb_lo ? g.dPb_lo + (size_t)m * g.ldy + n : nullptr, dp);
      } else {
        st16f(g.out + (size_t)m * g.ldo + n, v);
      }
    }
  }
  if (g.mode == kFitFwdLast) {
    if (h > 0) {
      s_e[2 * ((h - 1) * 128 + r)] = e_hi;
      s_e[2 * ((h - 1) * 128 + r) + 1] = e_lo;
    }
    __syncthreads();
    if (ok && h == 0 && valid) {
      for (int k = 1; k < WG; ++k) {
        comp_add(e_hi, e_lo, s_e[2 * ((k - 1) * 128 + r)]);
        e_lo += s_e[2 * ((k - 1) * 128 + r) + 1];
      }
      g.e_out[m] = ((double)e_hi + (double)e_lo) + (double)g.b_out[t];
    }
  }
  tc::fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tbase, kTmemCols);
}

// dE/dD of the first layer folded into dE/dxyz (FitDxyz).  One CTA per
// 128-row tile walks all 16 ng columns of dD in chunks of 128 (8 neurons),
// with its warps specialised: warp 4 loads (dP1 high and low BF16 parts once
// into shared memory, then W1 — per K chunk the high part, then the low
// part — through an S-stage TMA ring), warp 5 issues the MMAs of a chunk
// (the three split products dP hi . W hi, dP lo . W hi and dP hi . W lo
// summed in one accumulator; a W hi stage serves the first two) into one of
// two TMEM buffers, and
// warps 0-3 (thread = row) read the other buffer: the first term goes out
// per neuron, the transposed term of the first 16 neurons accumulates in
// registers and is added at the end.  The MMAs of chunk j + 1 run while the
// epilogue reads chunk j.
constexpr int kDxM = 16, kDxBN = 128, kDxStages = 5, kDxSeg = 2;
constexpr int kDxThreads = 192;  // 4 epilogue warps, the load warp, the MMA warp

__global__ void __launch_bounds__(kDxThreads, 1)
fit_dxyz_kernel(const __grid_constant__ CUtensorMap tma_a, const __grid_constant__ CUtensorMap tma_alo,
                const __grid_constant__ CUtensorMap tma_b, FitDxyz f, int* __restrict__ err) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char* smem = smem_raw + ((1024 - (tc::smem_u32(smem_raw) & 1023)) & 1023);
  constexpr int SA = 128 * kKC * 2, SB = kDxBN * kKC * 2, M = kDxM, S = kDxStages;
  __shared__ uint64_t full[S], empty[S], a_full, acc_full[2], acc_free[2], mma_done;
  __shared__ uint32_t s_tmem;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  int t = 0;
  while (t + 1 < f.ntypes && f.tile0[t + 1] <= (int)blockIdx.x) ++t;
  const int m0 = f.row0[t] + ((int)blockIdx.x - f.tile0[t]) * 128;
  const int rows_valid = min(128, f.row0[t + 1] - m0);
  const int ncol = f.ng * M, nk = (f.K + kKC - 1) / kKC, nchunk = (ncol + kDxBN - 1) / kDxBN;
  const int per = kDxSeg * nk;  // B loads of one column chunk: W hi over K, then W lo over K
  const int L = nchunk * per;   // B loads
  unsigned char* sA = smem;                // nk stages of dP1 (high part)
  unsigned char* sAlo = smem + nk * SA;    // nk stages of dP1 (low part)
  unsigned char* sB = smem + 2 * nk * SA;  // ring
  if (warp == 0) tc::tmem_alloc(&s_tmem, 2 * kDxBN);
  if (tid == 0) {
    for (int q = 0; q < S; ++q) {
      tc::mbar_init(&full[q], 1);
      tc::mbar_init(&empty[q], 1);
    }
    tc::mbar_init(&a_full, 1);
    for (int b = 0; b < 2; ++b) {
      tc::mbar_init(&acc_full[b], 1);
      tc::mbar_init(&acc_free[b], 4);  // one arrival per epilogue warp
    }
    tc::mbar_init(&mma_done, 1);
    tc::fence_mbar_init();
  }
  __syncthreads();
  tc::fence_after();
  const uint32_t tbase = s_tmem;
  bool ok = true;
  if (warp == 4) {
    if (lane == 0) {
      tc::mbar_expect_tx(&a_full, 2 * nk * SA);
      for (int k = 0; k < nk; ++k) {
        tc::tma_load_2d(tc::smem_u32(sA + k * SA), &tma_a, k * kKC, m0, &a_full);
        tc::tma_load_2d(tc::smem_u32(sAlo + k * SA), &tma_alo, k * kKC, m0, &a_full);
      }
      int next = 0;
      for (; next < L && ok; ++next) {
        const int q = next % S;
        if (next >= S) ok = tc::mbar_wait(&empty[q], ((next / S) - 1) & 1, err);
        if (!ok) break;
        const int j = next / per, rem = next - j * per, sg = rem / nk, k = rem - sg * nk;
        tc::mbar_expect_tx(&full[q], SB);
        tc::tma_load_2d(tc::smem_u32(sB + q * SB), &tma_b, (sg == 1 ? f.Kp : 0) + k * kKC, t * ncol + j * kDxBN,
                        &full[q]);
      }
      if (!ok) {
        // a wait ran out: let the copies already issued land before the CTA
        // ends (bounded; the most recent load of each stage)
        tc::mbar_wait(&a_full, 0, nullptr);
        for (int i = max(0, next - S); i < next; ++i) tc::mbar_wait(&full[i % S], (i / S) & 1, nullptr);
      }
    }
    __syncwarp();
  } else if (warp == 5) {
    if (lane == 0) {
      ok = tc::mbar_wait(&a_full, 0, err);
      for (int j = 0; j < nchunk && ok; ++j) {
        const int b = j & 1;
        // the epilogue has read chunk j - 2 out of this buffer
        if (j >= 2) ok = tc::mbar_wait(&acc_free[b], ((j >> 1) - 1) & 1, err);
        if (!ok) break;
        tc::fence_after();
        const int nt = min(kDxBN, ncol - j * kDxBN);  // 128 or a multiple of 16
        const uint32_t idesc = tc::idesc_bf16_f32(128, nt);
        const uint32_t dst = tbase + (uint32_t)(b * kDxBN);
        for (int u = 0; u < per && ok; ++u) {
          const int i = j * per + u, q = i % S, sg = u / nk, k = u - sg * nk;
          ok = tc::mbar_wait(&full[q], (i / S) & 1, err);
          if (!ok) break;
          tc::fence_after();
          const uint32_t a0 = tc::smem_u32(sA + k * SA), alo = tc::smem_u32(sAlo + k * SA);
          const uint32_t b0 = tc::smem_u32(sB + q * SB);
#pragma unroll
          for (int ks = 0; ks < kKC / 16; ++ks)
            tc::mma_bf16(dst, tc::smem_desc_sw128(a0 + ks * 32), tc::smem_desc_sw128(b0 + ks * 32), idesc,
                         (u > 0 || ks > 0) ? 1u : 0u);
          if (sg == 0)  // the same W hi stage with dP lo
#pragma unroll
            for (int ks = 0; ks < kKC / 16; ++ks)
              tc::mma_bf16(dst, tc::smem_desc_sw128(alo + ks * 32), tc::smem_desc_sw128(b0 + ks * 32), idesc, 1u);
          tc::mma_commit(&empty[q]);
        }
        tc::mma_commit(&acc_full[b]);
      }
      // every MMA issued has completed before the accumulator is freed
      tc::mma_commit(&mma_done);
      tc::mbar_wait(&mma_done, 0, nullptr);
    }
    __syncwarp();
  }
  // epilogue warps: the row's xyz[c][m < 16]; the transposed term of
  // neurons m < 16
  const int r = (warp & 3) * 32 + lane;
  const bool epi = warp < 4;
  const bool valid = epi && r < rows_valid;
  const int row = valid ? f.sorted_rows[m0 + r] : 0;
  const float* xr = f.xyz + (size_t)row * 4 * f.ng;
  float4* out = reinterpret_cast<float4*>(f.dxyz + (size_t)row * 4 * f.ng);
  float xm[4][M], T2[4][M];
#pragma unroll
  for (int c = 0; c < 4; ++c)
#pragma unroll
    for (int m = 0; m < M; ++m) {
      xm[c][m] = valid ? xr[c * f.ng + m] : 0.f;
      T2[c][m] = 0.f;
    }
  const float inv = 1.f / (float)f.nnei;
  constexpr int NH = kDxBN / M;  // neurons per chunk
  float xqn[NH][4];                // xyz[c][n] of the next chunk's neurons, in flight
  auto load_xq = [&](int j) {
    const int qn = j < nchunk ? min(kDxBN, ncol - j * kDxBN) / M : 0;
#pragma unroll
    for (int h = 0; h < NH; ++h)
#pragma unroll
      for (int c = 0; c < 4; ++c) xqn[h][c] = (valid && h < qn) ? xr[c * f.ng + j * NH + h] : 0.f;
  };
  if (epi) {
    load_xq(0);
    for (int j = 0; j < nchunk && ok; ++j) {
      const int b = j & 1;
      const int nt = min(kDxBN, ncol - j * kDxBN);
      const int q1 = nt / M;
      float xq[NH][4];
#pragma unroll
      for (int h = 0; h < NH; ++h)
#pragma unroll
        for (int c = 0; c < 4; ++c) xq[h][c] = xqn[h][c];
      load_xq(j + 1);
      ok = tc::mbar_wait(&acc_full[b], (j >> 1) & 1, err);
      ok = __all_sync(0xffffffffu, ok) != 0;  // the TMEM loads below are warp-wide
      if (!ok) break;
      tc::fence_after();
#pragma unroll
      for (int h = 0; h < NH; ++h) {
        const int q = h;
        if (q >= q1) break;
        const int n = j * NH + q;
        float v[16];
        tc::tmem_ld16(tc::taddr(tbase + (uint32_t)(b * kDxBN), (warp & 3) * 32, q * M), v);
        tc::tmem_ld_wait();
        if (!valid) continue;
        float t1[4], xn[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          float sacc = 0.f;
#pragma unroll
          for (int m = 0; m < M; ++m) sacc = fmaf(v[m], xm[c][m], sacc);
          t1[c] = sacc;
          xn[c] = xq[h][c];
        }
#pragma unroll
        for (int c = 0; c < 4; ++c)
#pragma unroll
          for (int m = 0; m < M; ++m) T2[c][m] = fmaf(v[m], xn[c], T2[c][m]);
        if (n < M)  // completed with the transposed term below
          out[n] = make_float4(t1[0], t1[1], t1[2], t1[3]);
        else
          out[n] = make_float4(t1[0] * inv, t1[1] * inv, t1[2] * inv, t1[3] * inv);
      }
      // this warp has read buffer b: the MMAs of chunk j + 2 may overwrite it
      tc::fence_before();
      __syncwarp();
      if (lane == 0) tc::mbar_arrive(&acc_free[b]);
    }
  }
  // the transposed term completes neurons m < 16
  ok = __syncthreads_and(ok) != 0;
  if (ok && valid)
#pragma unroll
    for (int m = 0; m < M; ++m) {
      const float4 a = out[m];
      out[m] = make_float4((a.x + T2[0][m]) * inv, (a.y + T2[1][m]) * inv, (a.z + T2[2][m]) * inv,
                           (a.w + T2[3][m]) * inv);
    }
  tc::fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tbase, 2 * kDxBN);
}

// cuTensorMapEncodeTiled, taken from the driver through the runtime
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

// bf16 matrix [rows, cols] with a row stride of ld elements, read in boxes of
// box_rows x 64 with 128-byte swizzling (out-of-range rows / columns read 0)
int encode_bf16_2d(CUtensorMap* m, const __nv_bfloat16* base, int rows, int cols, int ld, int box_rows) {
  PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
  if (!enc) return fail(DPGB_ECUDA, "cuTensorMapEncodeTiled is not available");
  if ((reinterpret_cast<uintptr_t>(base) & 15) || ((size_t)ld * 2) % 16)
    return fail(DPGB_EINVAL, "fitting GEMM operand not 16-byte aligned");
  const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
  const cuuint32_t box[2] = {(cuuint32_t)kKC, (cuuint32_t)box_rows};
  const cuuint32_t es[2] = {1, 1};
  const CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<__nv_bfloat16*>(base), dims, strides, box,
                         es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                         CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(DPGB_ECUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
  return DPGB_OK;
}

template <int BN, int S, int WG, int NA>
int launch_t(const FitGemm& g, int* err, cudaStream_t st) {
  const size_t smem = (size_t)S * (NA * 128 + 2 * BN) * kKC * 2 + 1024;  // + alignment slack
  static bool attr = false;
  if (!attr) {
    DPGB_CUDA(cudaFuncSetAttribute(fit_gemm_kernel<BN, S, WG, NA>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)smem));
    attr = true;
  }
  if (g.Kp < g.K || g.Kp % kKC || (NA == 2) != (g.A_lo != nullptr))
    return fail(DPGB_EINVAL, "fit_gemm: bad split-BF16 operands");
  CUtensorMap ta, talo, tb;
  DPGB_TRY(encode_bf16_2d(&ta, g.A, g.row0[g.ntypes], g.K, g.lda, 128));
  DPGB_TRY(encode_bf16_2d(&talo, g.A_lo ? g.A_lo : g.A, g.row0[g.ntypes], g.K, g.lda, 128));
  DPGB_TRY(encode_bf16_2d(&tb, g.B, g.ntypes * g.N, 2 * g.Kp, 2 * g.Kp, BN));
  // the column tiles of one row tile run next to each other (they read the
  // same A rows: L2 serves the repeats)
  dim3 grid(ceil_div(g.N, BN), g.tile0[g.ntypes]);
  fit_gemm_kernel<BN, S, WG, NA><<<grid, 128 * WG, smem, st>>>(ta, talo, tb, g, err);
  return check_launch("fit_gemm");
}

}  // namespace

int fit_tc_eligible(const dpgb_se_a_desc& d) {
  if (d.dim_descrpt % 16 || d.ntypes > 8) return 0;
  int nin = d.dim_descrpt;
  for (int l = 0; l < d.n_fit; ++l) {
    const int w = d.fit_neuron[l];
    if (w % 16 || w > 256) return 0;
    if (w == 2 * nin) return 0;  // the doubling skip is not fused here
    nin = w;
  }
  return d.n_fit >= 1;
}

int launch_fit_dxyz(const FitDxyz& f, int* err, cudaStream_t st) {
  if (f.tile0[f.ntypes] <= 0) return DPGB_OK;
  const int nk = (f.K + kKC - 1) / kKC;
  const size_t smem = (size_t)2 * nk * 128 * kKC * 2 + (size_t)kDxStages * kDxBN * kKC * 2 + 1024;
  if (smem > 227 * 1024) return fail(DPGB_EINVAL, "fit_dxyz: first hidden layer too wide");
  if (f.Kp != nk * kKC || !f.A_lo) return fail(DPGB_EINVAL, "fit_dxyz: bad split-BF16 operands");
  DPGB_CUDA(cudaFuncSetAttribute(fit_dxyz_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  CUtensorMap ta, talo, tb;
  DPGB_TRY(encode_bf16_2d(&ta, f.A, f.row0[f.ntypes], f.K, f.lda, 128));
  DPGB_TRY(encode_bf16_2d(&talo, f.A_lo, f.row0[f.ntypes], f.K, f.lda, 128));
  DPGB_TRY(encode_bf16_2d(&tb, f.B, f.ntypes * f.ng * kDxM, 2 * f.Kp, 2 * f.Kp, kDxBN));
  fit_dxyz_kernel<<<f.tile0[f.ntypes], kDxThreads, smem, st>>>(ta, talo, tb, f, err);
  return check_launch("fit_dxyz");
}

int launch_fit_gemm(const FitGemm& g, int* err, cudaStream_t st) {
  const int mt = g.tile0[g.ntypes];
  if (mt <= 0) return DPGB_OK;
  // stages: three when two CTAs still fit on an SM, else two
  const bool split_a = g.A_lo != nullptr;
  if (g.mode == kFitFwdLast)  // the output layer needs whole rows (one CTA per SM)
    return split_a ? launch_t<256, 2, 2, 2>(g, err, st) : launch_t<256, 2, 2, 1>(g, err, st);
  // column tile: the narrower one when it spreads the tiles more evenly over
  // the SMs (two CTAs fit on an SM either way): for 240 columns, three
  // 80-wide tiles per row tile rather than a 128 + 112 pair
  const int sms = sm_count();
  auto span = [&](int bn) { return (long long)ceil_div(mt * ceil_div(g.N, bn), 2 * sms) * bn; };
  if (g.N % 80 == 0 && span(80) < span(128))
    return split_a ? launch_t<80, 2, 2, 2>(g, err, st) : launch_t<80, 3, 2, 1>(g, err, st);
  return split_a ? launch_t<128, 2, 2, 2>(g, err, st) : launch_t<128, 2, 2, 1>(g, err, st);
}

}  // namespace dpgb
