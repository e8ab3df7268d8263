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

#include <algorithm>

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
  // both forms, then a select: no branch per element in the epilogues
  const float a = fabsf(x);
  const float x2 = x * x;
  const float ser = x * fmaf(x2, fmaf(x2, fmaf(x2, -17.f / 315.f, 2.f / 15.f), -1.f / 3.f), 1.f);
  const float e = __expf(2.f * fminf(a, 12.f));
  const float big = copysignf(1.f - __fdividef(2.f, e + 1.f), x);
  return a < 0.0625f ? ser : big;
}

// high and low BF16 parts of an FP32 value (hi + lo carries ~16 bits)
__device__ __forceinline__ void split_bf16(float v, __nv_bfloat16& hi, __nv_bfloat16& lo) {
  hi = __float2bfloat16_rn(v);
  lo = __float2bfloat16_rn(v - __bfloat162float(hi));
}


// --- epilogue staging -------------------------------------------------------
// Each epilogue warp owns a 2 KB tile of shared memory through which its 32
// rows x 16 columns pass between the thread-per-row layout of the
// accumulator and coalesced global accesses (a warp instruction then covers
// 8 rows x 64 bytes of FP32, or 16 rows x 32 bytes of BF16, instead of 32
// rows x 16 bytes).  FP32 tile: row r, 16-byte chunk c at unit
// 4 r + (c ^ ((r >> 1) & 3)); BF16 tile: unit 2 r + (c ^ ((r >> 2) & 1)).
// Both the row-wise and the coalesced patterns are then free of bank
// conflicts.
constexpr int kStageFloats = 32 * 16;  // one warp's tile

__device__ __forceinline__ int unit_f32(int r, int c) { return 4 * r + (c ^ ((r >> 1) & 3)); }
__device__ __forceinline__ int unit_b16(int r, int c) { return 2 * r + (c ^ ((r >> 2) & 1)); }

// this thread's row (lane) of 16 floats into / out of the tile
__device__ __forceinline__ void put_row(float4* w, int lane, const float (&v)[16]) {
#pragma unroll
  for (int c = 0; c < 4; ++c) w[unit_f32(lane, c)] = make_float4(v[4 * c], v[4 * c + 1], v[4 * c + 2], v[4 * c + 3]);
}
__device__ __forceinline__ void get_row(const float4* w, int lane, float (&v)[16]) {
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    const float4 x = w[unit_f32(lane, c)];
    v[4 * c] = x.x;
    v[4 * c + 1] = x.y;
    v[4 * c + 2] = x.z;
    v[4 * c + 3] = x.w;
  }
}
// coalesced: the lane's (row (lane >> 2) + 8 k, chunk lane & 3), k = 0..3, of
// the warp's rows starting at base (row stride ld floats); rows >= rows_ok
// are neither read (zeros) nor written
__device__ __forceinline__ void load_tile(float4 (&x)[4], int lane, const float* base, size_t ld, int rows_ok) {
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int r = (lane >> 2) + 8 * k;
    x[k] = r < rows_ok ? *reinterpret_cast<const float4*>(base + (size_t)r * ld + 4 * (lane & 3))
                       : make_float4(0.f, 0.f, 0.f, 0.f);
  }
}
__device__ __forceinline__ void put_tile(float4* w, int lane, const float4 (&x)[4]) {
#pragma unroll
  for (int k = 0; k < 4; ++k) w[unit_f32((lane >> 2) + 8 * k, lane & 3)] = x[k];
}
__device__ __forceinline__ void store_tile(const float4* w, int lane, float* base, size_t ld, int rows_ok) {
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int r = (lane >> 2) + 8 * k;
    if (r < rows_ok) *reinterpret_cast<float4*>(base + (size_t)r * ld + 4 * (lane & 3)) = w[unit_f32(r, lane & 3)];
  }
}
// BF16: the row's 16 values split once into high parts (units 0..63 of the
// tile) and low parts (units 64..127), then stored coalesced
__device__ __forceinline__ void put_row_b16(float4* w, int lane, const float (&v)[16]) {
  __nv_bfloat162 h[8], l[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    __nv_bfloat16 a, b, al, bl;
    split_bf16(v[2 * i], a, al);
    split_bf16(v[2 * i + 1], b, bl);
    h[i] = __halves2bfloat162(a, b);
    l[i] = __halves2bfloat162(al, bl);
  }
  uint4* u = reinterpret_cast<uint4*>(w);
  u[unit_b16(lane, 0)] = *reinterpret_cast<const uint4*>(&h[0]);
  u[unit_b16(lane, 1)] = *reinterpret_cast<const uint4*>(&h[4]);
  u[64 + unit_b16(lane, 0)] = *reinterpret_cast<const uint4*>(&l[0]);
  u[64 + unit_b16(lane, 1)] = *reinterpret_cast<const uint4*>(&l[4]);
}
__device__ __forceinline__ void store_tile_b16(const float4* w, int lane, __nv_bfloat16* base, size_t ld,
                                               int rows_ok) {
  const uint4* u = reinterpret_cast<const uint4*>(w);
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const int r = (lane >> 1) + 16 * k;
    if (r < rows_ok) *reinterpret_cast<uint4*>(base + (size_t)r * ld + 8 * (lane & 1)) = u[unit_b16(r, lane & 1)];
  }
}

// FP32 values of this thread's row through the tile to global memory
__device__ __forceinline__ void emit_f32(float4* w, int lane, const float (&v)[16], float* base, size_t ld,
                                         int rows_ok) {
  put_row(w, lane, v);
  __syncwarp();
  store_tile(w, lane, base, ld, rows_ok);
  __syncwarp();
}
// two FP32 rows through two tiles with one exchange (w2 == w: one after the other)
__device__ __forceinline__ void emit2_f32(float4* w, float4* w2, int lane, const float (&a)[16], float* base_a,
                                          const float (&b)[16], float* base_b, size_t ld, int rows_ok) {
  if (w2 == w) {
    emit_f32(w, lane, a, base_a, ld, rows_ok);
    emit_f32(w, lane, b, base_b, ld, rows_ok);
    return;
  }
  put_row(w, lane, a);
  put_row(w2, lane, b);
  __syncwarp();
  store_tile(w, lane, base_a, ld, rows_ok);
  store_tile(w2, lane, base_b, ld, rows_ok);
  __syncwarp();
}
// split BF16 (hi at base, lo at base_lo when set)
__device__ __forceinline__ void emit_b16(float4* w, int lane, const float (&v)[16], __nv_bfloat16* base,
                                         __nv_bfloat16* base_lo, size_t ld, int rows_ok) {
  put_row_b16(w, lane, v);
  __syncwarp();
  store_tile_b16(w, lane, base, ld, rows_ok);
  if (base_lo) store_tile_b16(w + 64, lane, base_lo, ld, rows_ok);
  __syncwarp();
}

// Per-type column vectors of the epilogue, staged in shared memory at the
// start of the kernel: [type][3][N] floats —
//   forward: bias, idt (1 when absent), w_out (output layer);
//   backward: idt of the lower layer (1 when absent), the broadcast upstream
//   gradient (dYup with lddyup == 0; 0 when absent), unused.
__device__ __forceinline__ float fit_vec(const FitGemm& g, int t, int a, int n) {
  const size_t o = (size_t)t * g.N + n;
  if (g.mode == kFitBwd) {
    if (a == 0) return g.idt_lo ? g.idt_lo[o] : 1.f;
    if (a == 1) return (g.dYup && g.lddyup == 0) ? g.dYup[o] : 0.f;
    return 0.f;
  }
  if (a == 0) return g.bias ? g.bias[o] : 0.f;
  if (a == 1) return g.idt ? g.idt[o] : 1.f;
  return g.w_out ? g.w_out[o] : 0.f;
}
// work item -> type, first row, first column (nnt column tiles per row tile)
__device__ __forceinline__ void fit_decode(const FitGemm& g, int BN, int nnt, int it, int& t, int& m0, int& n0) {
  const int tile = it / nnt;
  n0 = (it - tile * nnt) * BN;
  t = 0;
  while (t + 1 < g.ntypes && g.tile0[t + 1] <= tile) ++t;
  m0 = g.row0[t] + (tile - g.tile0[t]) * 128;
}

// The epilogue warps' part of fit_gemm_kernel for one mode: this warp (of
// group h, TMEM quadrant q) walks the items j = h (mod EG) of the CTA, 16
// accumulator columns at a time.
template <int MODE, int BN, int EG, int NB, uint32_t kCols>
__device__ __forceinline__ void fit_epilogue(const FitGemm& g, const float* svec, float4* wst, float4* wst2,
                                             uint32_t tbase, uint64_t* acc_full, uint64_t* acc_free, int* err) {
  constexpr bool fwd = MODE == kFitFwd || MODE == kFitFwdLast, bwd = MODE == kFitBwd;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, h = warp >> 2, q = warp & 3;
  const int nnt = (g.N + BN - 1) / BN, items = g.tile0[g.ntypes] * nnt;
  const bool in_a = (fwd && g.skip) || (bwd && g.dYup && g.lddyup);  // row operands
  const float* xa = fwd ? g.Xs : g.dYup;
  const size_t lda_in = fwd ? (size_t)g.ldxs : (size_t)g.lddyup;
  int j = h;
  for (int it = blockIdx.x + h * gridDim.x; it < items; it += EG * gridDim.x, j += EG) {
    const int b = j % NB;
    int t, m0, n0;
    fit_decode(g, BN, nnt, it, t, m0, n0);
    const int mw = m0 + q * 32;                      // the warp's first row
    const int rows_ok = min(32, g.row0[t + 1] - mw);  // its rows of type t
    const int nt = min(BN, g.N - n0);
    const float* vec = svec + (size_t)t * 3 * g.N;
    float4 pa[4], pb[4];  // the next 16 columns' row operands (coalesced)
    if (in_a) load_tile(pa, lane, xa + (size_t)mw * lda_in + n0, lda_in, rows_ok);
    if (bwd) load_tile(pb, lane, g.T_lo + (size_t)mw * g.ldy + n0, g.ldy, rows_ok);
    bool ok = tc::mbar_wait(&acc_full[b], (j / NB) & 1, err);
    ok = __all_sync(0xffffffffu, ok) != 0;  // the TMEM loads below are warp-wide
    if (!ok) break;
    tc::fence_after();
    float e_hi = 0.f, e_lo = 0.f;  // output layer: compensated sum of y w over the row
    for (int c0 = 0; c0 < nt; c0 += 16) {
      const int n = n0 + c0;
      float xa_r[16], xb_r[16];
      if (in_a && bwd && wst2 != wst) {  // both row operands through the two tiles at once
        put_tile(wst, lane, pa);
        put_tile(wst2, lane, pb);
        __syncwarp();
        get_row(wst, lane, xa_r);
        get_row(wst2, lane, xb_r);
        __syncwarp();
      } else {
        if (in_a) {
          put_tile(wst, lane, pa);
          __syncwarp();
          get_row(wst, lane, xa_r);
          __syncwarp();
        }
        if (bwd) {
          put_tile(wst, lane, pb);
          __syncwarp();
          get_row(wst, lane, xb_r);
          __syncwarp();
        }
      }
      if (c0 + 16 < nt) {
        if (in_a) load_tile(pa, lane, xa + (size_t)mw * lda_in + n + 16, lda_in, rows_ok);
        if (bwd) load_tile(pb, lane, g.T_lo + (size_t)mw * g.ldy + n + 16, g.ldy, rows_ok);
      }
      float v[16];
      tc::tmem_ld16(tc::taddr(tbase + (uint32_t)(b * kCols), q * 32, c0), v);
      tc::tmem_ld_wait();
      if (fwd) {
        float tv[16];
        const float4* bb = reinterpret_cast<const float4*>(vec + n);
        const float4* id = reinterpret_cast<const float4*>(vec + g.N + n);
#pragma unroll
        for (int i4 = 0; i4 < 4; ++i4) {
          const float4 b4 = bb[i4], d4 = id[i4];
          const float bv[4] = {b4.x, b4.y, b4.z, b4.w}, dv[4] = {d4.x, d4.y, d4.z, d4.w};
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const int i = 4 * i4 + u;
            tv[i] = tanh_acc(v[i] + bv[u]);
            v[i] = tv[i] * dv[u];  // y
            if (in_a) v[i] += xa_r[i];
          }
        }
        if (MODE == kFitFwd) {
          emit2_f32(wst, wst2, lane, v, g.Yf + (size_t)mw * g.ldy + n, tv, g.Tt + (size_t)mw * g.ldy + n, g.ldy,
                    rows_ok);
          emit_b16(wst, lane, v, g.Yb + (size_t)mw * g.ldy + n, g.Yb_lo ? g.Yb_lo + (size_t)mw * g.ldy + n : nullptr,
                   g.ldy, rows_ok);
        } else {
          const float4* wo = reinterpret_cast<const float4*>(vec + 2 * g.N + n);
#pragma unroll
          for (int i4 = 0; i4 < 4; ++i4) {
            const float4 w4 = wo[i4], d4 = id[i4];
            const float wv[4] = {w4.x, w4.y, w4.z, w4.w}, dv[4] = {d4.x, d4.y, d4.z, d4.w};
#pragma unroll
            for (int u = 0; u < 4; ++u) {
              const int i = 4 * i4 + u;
              const float pr = v[i] * wv[u];
              comp_add(e_hi, e_lo, pr);
              e_lo += fmaf(v[i], wv[u], -pr);                  // the product's rounding error
              tv[i] = wv[u] * dv[u] * (1.f - tv[i] * tv[i]);  // dP
            }
          }
          emit_b16(wst, lane, tv, g.dPb + (size_t)mw * g.ldy + n,
                   g.dPb_lo ? g.dPb_lo + (size_t)mw * g.ldy + n : nullptr, g.ldy, rows_ok);
        }
      } else if (bwd) {
        const float* il = vec + n;
        const float* up = vec + g.N + n;
#pragma unroll
        for (int i = 0; i < 16; ++i) v[i] += in_a ? xa_r[i] : up[i];  // dx (up is 0 without dYup)
        if (g.dXf) emit_f32(wst, lane, v, g.dXf + (size_t)mw * g.ldy + n, g.ldy, rows_ok);
#pragma unroll
        for (int i = 0; i < 16; ++i) v[i] = v[i] * il[i] * (1.f - xb_r[i] * xb_r[i]);  // dP
        emit_b16(wst, lane, v, g.dPb + (size_t)mw * g.ldy + n, g.dPb_lo ? g.dPb_lo + (size_t)mw * g.ldy + n : nullptr,
                 g.ldy, rows_ok);
      } else {
        emit_f32(wst, lane, v, g.out + (size_t)mw * g.ldo + n, g.ldo, rows_ok);
      }
    }
    // this warp has read the buffer: the MMAs of item j + NB may overwrite it
    tc::fence_before();
    __syncwarp();
    if (lane == 0) tc::mbar_arrive(&acc_free[b]);
    if (MODE == kFitFwdLast && lane < rows_ok) g.e_out[mw + lane] = ((double)e_hi + (double)e_lo) + (double)g.b_out[t];
  }
}

// Persistent, warp-specialised GEMM: the CTA (one per SM) walks the work
// items it, it + gridDim.x, ... (an item: one 128-row tile by one BN-column
// tile).  Warp 4 EG streams the items' K chunks through an S-stage TMA
// ring, warp 4 EG + 1 issues their MMAs into one of NB TMEM accumulators
// (item j of the CTA into buffer j mod NB), and each of the EG epilogue warp
// groups (warps 4h .. 4h + 3, thread = row) runs the epilogue of the items
// j = h (mod EG): the MMAs of the next items overlap the epilogue of item j,
// and the groups' epilogues overlap each other.  The epilogue reads its row
// operands (skip input, upstream gradient, tanh values) and writes its
// outputs through its warp's staging tile, 16 columns at a time, with the
// next 16 columns' operands in flight.
// NA: parts of A (1: hi, 2: hi and lo); the weight always comes as hi and
// lo.  A stage holds one K chunk of every part, so each part is read once.
template <int BN, int S, int NA, int EG, int NB, int TILES>
__global__ void __launch_bounds__(128 * EG + 64, 1)
fit_gemm_kernel(const __grid_constant__ CUtensorMap tma_a, const __grid_constant__ CUtensorMap tma_alo,
                const __grid_constant__ CUtensorMap tma_b, FitGemm g, int* __restrict__ err) {
  extern __shared__ unsigned char smem_raw[];
  // swizzled TMA tiles want 1024-byte aligned stages
  unsigned char* smem = smem_raw + ((1024 - (tc::smem_u32(smem_raw) & 1023)) & 1023);
  __shared__ uint64_t full[S], empty[S], acc_full[NB], acc_free[NB], mma_done;
  __shared__ uint32_t s_tmem;
  constexpr int SA = 128 * kKC * 2, SB = BN * kKC * 2, STAGE = NA * SA + 2 * SB;
  constexpr uint32_t kCols = BN <= 32 ? 32 : (BN <= 64 ? 64 : (BN <= 128 ? 128 : 256));  // a buffer's columns
  static_assert(BN % 16 == 0 && BN <= 256 && SB % 1024 == 0, "whole 16-column loads, 1024-byte aligned stages");
  // the allocation: a power of two of at least NB buffers
  constexpr uint32_t kAlloc = NB * kCols <= 128 ? 128 : (NB * kCols <= 256 ? 256 : 512);
  static_assert(NB * kCols <= 512, "TMEM: 512 columns per SM");
  float4* stage_tiles = reinterpret_cast<float4*>(smem + S * STAGE);  // TILES per epilogue warp
  float* svec = reinterpret_cast<float*>(smem + S * STAGE + TILES * EG * 4 * kStageFloats * 4);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nnt = (g.N + BN - 1) / BN, items = g.tile0[g.ntypes] * nnt;
  const int nchunk = (g.K + kKC - 1) / kKC;
  if (warp == 0) tc::tmem_alloc(&s_tmem, kAlloc);
  if (tid == 0) {
    for (int s = 0; s < S; ++s) {
      tc::mbar_init(&full[s], 1);
      tc::mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < NB; ++b) {
      tc::mbar_init(&acc_full[b], 1);
      tc::mbar_init(&acc_free[b], 4);  // one arrival per warp of the reading warp group
    }
    tc::mbar_init(&mma_done, 1);
    tc::fence_mbar_init();
  }
  for (int q = tid; q < g.ntypes * 3 * g.N; q += blockDim.x) {
    const int t = q / (3 * g.N), rem = q - t * 3 * g.N, a = rem / g.N;
    svec[q] = fit_vec(g, t, a, rem - a * g.N);
  }
  __syncthreads();
  tc::fence_after();
  const uint32_t tbase = s_tmem;
  bool ok = true;
  if (warp == 4 * EG) {
    if (lane == 0) {
      // producer: the c-th chunk of the CTA into stage c % S once the MMAs
      // of chunk c - S released it (stage layout: A hi [, A lo], B hi, B lo)
      int c = 0;
      for (int it = blockIdx.x; it < items && ok; it += gridDim.x) {
        int t, m0, n0;
        fit_decode(g, BN, nnt, it, t, m0, n0);
        for (int i = 0; i < nchunk; ++i, ++c) {
          const int s = c % S;
          if (c >= S) ok = tc::mbar_wait(&empty[s], ((c / S) - 1) & 1, err);
          if (!ok) break;
          const uint32_t a0 = tc::smem_u32(smem + s * STAGE), b0 = a0 + NA * SA;
          tc::mbar_expect_tx(&full[s], STAGE);
          tc::tma_load_2d(a0, &tma_a, i * kKC, m0, &full[s]);
          if (NA == 2) tc::tma_load_2d(a0 + SA, &tma_alo, i * kKC, m0, &full[s]);
          tc::tma_load_2d(b0, &tma_b, i * kKC, t * g.N + n0, &full[s]);
          tc::tma_load_2d(b0 + SB, &tma_b, g.Kp + i * kKC, t * g.N + n0, &full[s]);
        }
      }
      if (!ok)  // a wait ran out: the copies already issued land before the CTA ends (bounded)
        for (int i = max(0, c - S); i < c; ++i) tc::mbar_wait(&full[i % S], (i / S) & 1, nullptr);
    }
    __syncwarp();
  } else if (warp == 4 * EG + 1) {
    if (lane == 0) {
      // MMA issuer: 4 steps of K = 16 per chunk (zeros past K add nothing),
      // each hi.hi (+ lo.hi) + hi.lo
      int c = 0, j = 0;
      for (int it = blockIdx.x; it < items && ok; it += gridDim.x, ++j) {
        int t, m0, n0;
        fit_decode(g, BN, nnt, it, t, m0, n0);
        const int b = j % NB;
        // the epilogue has read item j - NB out of this buffer
        if (j >= NB) ok = tc::mbar_wait(&acc_free[b], ((j / NB) - 1) & 1, err);
        if (!ok) break;
        tc::fence_after();
        const uint32_t idesc = tc::idesc_bf16_f32(128, min(BN, g.N - n0));
        const uint32_t dst = tbase + (uint32_t)(b * kCols);
        for (int i = 0; i < nchunk && ok; ++i, ++c) {
          const int s = c % S;
          ok = tc::mbar_wait(&full[s], (c / S) & 1, err);
          if (!ok) break;
          tc::fence_after();
          const uint32_t a0 = tc::smem_u32(smem + s * STAGE), b0 = a0 + NA * SA;
#pragma unroll
          for (int ks = 0; ks < kKC / 16; ++ks) {
            tc::mma_bf16(dst, tc::smem_desc_sw128(a0 + ks * 32), tc::smem_desc_sw128(b0 + ks * 32), idesc,
                         (i > 0 || ks > 0) ? 1u : 0u);
            if (NA == 2)
              tc::mma_bf16(dst, tc::smem_desc_sw128(a0 + SA + ks * 32), tc::smem_desc_sw128(b0 + ks * 32), idesc,
                           1u);
            tc::mma_bf16(dst, tc::smem_desc_sw128(a0 + ks * 32), tc::smem_desc_sw128(b0 + SB + ks * 32), idesc, 1u);
          }
          tc::mma_commit(&empty[s]);
        }
        if (ok) tc::mma_commit(&acc_full[b]);
      }
      // every MMA issued has completed before the accumulators are freed
      tc::mma_commit(&mma_done);
      tc::mbar_wait(&mma_done, 0, nullptr);
    }
    __syncwarp();
  } else {
    // epilogue: warp group h takes the CTA's items j = h, h + EG, ...
    // (buffer j mod NB); thread = row (warp quadrant q = TMEM lanes 32 q ..)
    float4* wst = stage_tiles + TILES * warp * (kStageFloats / 4);
    float4* wst2 = TILES == 2 ? wst + kStageFloats / 4 : wst;
    switch (g.mode) {
      case kFitFwd:
        fit_epilogue<kFitFwd, BN, EG, NB, kCols>(g, svec, wst, wst2, tbase, acc_full, acc_free, err);
        break;
      case kFitFwdLast:
        fit_epilogue<kFitFwdLast, BN, EG, NB, kCols>(g, svec, wst, wst2, tbase, acc_full, acc_free, err);
        break;
      case kFitBwd:
        fit_epilogue<kFitBwd, BN, EG, NB, kCols>(g, svec, wst, wst2, tbase, acc_full, acc_free, err);
        break;
      default: fit_epilogue<kFitStore, BN, EG, NB, kCols>(g, svec, wst, wst2, tbase, acc_full, acc_free, err); break;
    }
  }
  tc::fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tbase, kAlloc);
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
constexpr int kDxM = 16, kDxBN = 128, kDxStages = 4, kDxSeg = 2;
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
  // neurons m < 16 in (even, odd) pairs, for the packed FP32 FMA (two IEEE
  // fmaf results per instruction)
  float2 xm[4][M / 2], T2[4][M / 2];
#pragma unroll
  for (int c = 0; c < 4; ++c)
#pragma unroll
    for (int k = 0; k < M / 2; ++k) {
      xm[c][k] = valid ? make_float2(xr[c * f.ng + 2 * k], xr[c * f.ng + 2 * k + 1]) : make_float2(0.f, 0.f);
      T2[c][k] = make_float2(0.f, 0.f);
    }
  const float inv = 1.f / (float)f.nnei;
  constexpr int NH = kDxBN / M;  // neurons per chunk
  float xqn[NH][4];                // xyz[c][n] of the next chunk's neurons, in flight
  const bool vec4 = (f.ng & 3) == 0;  // the chunk's neurons of a component as 16-byte aligned float4 pairs
  auto load_xq = [&](int j) {
    const int qn = j < nchunk ? min(kDxBN, ncol - j * kDxBN) / M : 0;
    if (vec4) {
#pragma unroll
      for (int c = 0; c < 4; ++c)
#pragma unroll
        for (int h4 = 0; h4 < NH; h4 += 4) {
          const float4 x = (valid && h4 < qn) ? *reinterpret_cast<const float4*>(xr + c * f.ng + j * NH + h4)
                                              : make_float4(0.f, 0.f, 0.f, 0.f);
          xqn[h4][c] = x.x;
          xqn[h4 + 1][c] = x.y;
          xqn[h4 + 2][c] = x.z;
          xqn[h4 + 3][c] = x.w;
        }
      return;
    }
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
        float2 v2[M / 2];
#pragma unroll
        for (int k = 0; k < M / 2; ++k) v2[k] = make_float2(v[2 * k], v[2 * k + 1]);
        float t1[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          // two interleaved chains of M / 2, even and odd m (eight independent chains with c)
          float2 s01 = make_float2(0.f, 0.f);
#pragma unroll
          for (int k = 0; k < M / 2; ++k) s01 = __ffma2_rn(v2[k], xm[c][k], s01);
          t1[c] = s01.x + s01.y;
        }
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          const float2 xn = make_float2(xq[h][c], xq[h][c]);
#pragma unroll
          for (int k = 0; k < M / 2; ++k) T2[c][k] = __ffma2_rn(v2[k], xn, T2[c][k]);
        }
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
      auto t2 = [&](int c) { return (m & 1) ? T2[c][m >> 1].y : T2[c][m >> 1].x; };
      out[m] = make_float4((a.x + t2(0)) * inv, (a.y + t2(1)) * inv, (a.z + t2(2)) * inv, (a.w + t2(3)) * inv);
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

// epilogue shared memory next to the stages: the warps' staging tiles and
// the per-type column vectors
constexpr size_t epi_bytes(int EG, int tiles, int ntypes, int N) {
  return (size_t)tiles * EG * 4 * kStageFloats * 4 + (size_t)ntypes * 3 * N * 4;
}

// stages of a BN-column tile: as many as fit next to each other and the
// epilogue's shared memory (one tile per warp, up to two types of 256
// columns) in about 220 KB (2 .. 6)
template <int BN, int NA, int EG>
constexpr int fit_stages() {
  constexpr int stage = (NA * 128 + 2 * BN) * kKC * 2;
  constexpr int s = (int)((220 * 1024 - epi_bytes(EG, 1, 2, 256)) / stage);
  return s < 2 ? 2 : (s > 6 ? 6 : s);
}

template <int BN, int NA, int EG, int NB, int TILES>
int launch_tiles(const FitGemm& g, int* err, cudaStream_t st, size_t smem) {
  constexpr int S = fit_stages<BN, NA, EG>();
  static size_t attr = 0;  // the largest dynamic shared memory requested so far
  if (attr < smem) {
    DPGB_CUDA(cudaFuncSetAttribute(fit_gemm_kernel<BN, S, NA, EG, NB, TILES>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr = smem;
  }
  CUtensorMap ta, talo, tb;
  DPGB_TRY(encode_bf16_2d(&ta, g.A, g.row0[g.ntypes], g.K, g.lda, 128));
  DPGB_TRY(encode_bf16_2d(&talo, g.A_lo ? g.A_lo : g.A, g.row0[g.ntypes], g.K, g.lda, 128));
  DPGB_TRY(encode_bf16_2d(&tb, g.B, g.ntypes * g.N, 2 * g.Kp, 2 * g.Kp, BN));
  const int items = g.tile0[g.ntypes] * ceil_div(g.N, BN);
  fit_gemm_kernel<BN, S, NA, EG, NB, TILES><<<std::min(items, sm_count()), 128 * EG + 64, smem, st>>>(ta, talo, tb,
                                                                                                     g, err);
  return check_launch("fit_gemm");
}

template <int BN, int NA, int EG, int NB>
int launch_t(const FitGemm& g, int* err, cudaStream_t st) {
  constexpr int S = fit_stages<BN, NA, EG>();
  if (g.Kp < g.K || g.Kp % kKC || (NA == 2) != (g.A_lo != nullptr))
    return fail(DPGB_EINVAL, "fit_gemm: bad split-BF16 operands");
  if (g.mode == kFitFwdLast && g.N > BN) return fail(DPGB_EINVAL, "fit_gemm: the output layer needs whole rows");
  // + alignment slack; at least half of an SM's shared memory, so that one
  // CTA (and its TMEM accumulators) sits on an SM.  Two staging tiles per
  // epilogue warp where they fit (fewer exchanges per 16 columns), else one.
  auto bytes = [&](int tiles) {
    return std::max((size_t)S * (NA * 128 + 2 * BN) * kKC * 2 + 1024 + epi_bytes(EG, tiles, g.ntypes, g.N),
                    (size_t)116 * 1024);
  };
  constexpr size_t kMax = 226 * 1024;
  if (bytes(2) <= kMax) return launch_tiles<BN, NA, EG, NB, 2>(g, err, st, bytes(2));
  if (bytes(1) <= kMax) return launch_tiles<BN, NA, EG, NB, 1>(g, err, st, bytes(1));
  return fail(DPGB_EINVAL, "fit_gemm: too many atom types for the staged epilogue");
}

template <int NA>
int launch_na(const FitGemm& g, int* err, cudaStream_t st) {
  // Row tiles that give every SM two items or more: 128-column items in the
  // forward hidden layers, whole rows (two accumulators) in the output
  // layer and the backward; fewer: 80- (or 64-) column items spread the
  // rows' work over more SMs.
  const int rows_tiles = g.tile0[g.ntypes];
  const bool enough = g.mode == kFitFwdLast || (long long)rows_tiles * ceil_div(g.N, 256) >= 2LL * sm_count();
  if (!enough) {
    if (g.N % 80 == 0) return launch_t<80, NA, 2, 4>(g, err, st);
    return launch_t<64, NA, 2, 4>(g, err, st);
  }
  if (g.N <= 64) return launch_t<64, NA, 2, 4>(g, err, st);
  // the forward hidden layers: column tiles of 128 with four accumulators,
  // so that the MMAs run ahead of both epilogue groups (measured faster
  // there); the output layer and the backward keep whole rows
  if (g.N <= 128 || g.mode == kFitFwd) return launch_t<128, NA, 2, 4>(g, err, st);
  if (g.N <= 240) return launch_t<240, NA, 2, 2>(g, err, st);
  return launch_t<256, NA, 2, 2>(g, err, st);
}

}  // namespace

int fit_tc_eligible(const dpgb_se_a_desc& d) {
  if (d.dim_descrpt % 16 || d.ntypes > 8) return 0;
  int nin = d.dim_descrpt;
  for (int l = 0; l < d.n_fit; ++l) {
    const int w = d.fit_neuron[l];
    if (w % 16 || w > 256) return 0;
    if (w > 240 && d.ntypes > 4) return 0;  // the epilogue's shared memory
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
  if (g.tile0[g.ntypes] <= 0) return DPGB_OK;
  if (g.N % 16) return fail(DPGB_EINVAL, "fit_gemm: width not a multiple of 16");
  return g.A_lo ? launch_na<2>(g, err, st) : launch_na<1>(g, err, st);
}

}  // namespace dpgb
