// Compressed se_e2_a descriptor for the mixed-precision DeepPot: the table
// lookup of tabulate_fusion_se_a (source/lib/src/gpu/tabulate.cu:293-506)
// fused with the environment matrix, the G^T R~ contraction, D, and on the
// way back the pair gradients and per-atom virial — on the CUDA cores in FP32
// (the table is a per-interval quintic: no GEMM to give the tensor cores).
// The work decomposition is described above the kernels.
#include <cuda_bf16.h>

#include <algorithm>

#include "emb_tc.cuh"
#include "se_a.cuh"

namespace dpgb {
namespace {

// a hint: move the 128-byte line holding p into L2 (global memory)
__device__ __forceinline__ void prefetch_l2(const void* p) {
  asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

struct SlotEnv {
  int nb;        // extended index, -1 padding
  int active;    // contributes to xyz
  float rn[4];   // normalised R~
  float d[3];    // r_j - r_i (FP32 of the FP64 difference)
  int idx;       // table interval
  float xx, delta;
};

__device__ __forceinline__ float switch_f(float nr, float rmin, float rmax, float& dsw) {
  if (nr < rmin) {
    dsw = 0.f;
    return 1.f;
  }
  if (nr < rmax) {
    const float du = 1.f / (rmax - rmin);
    const float uu = (nr - rmin) * du;
    const float poly = -6.f * uu * uu + 15.f * uu - 10.f;
    dsw = (3.f * uu * uu * poly + uu * uu * uu * (-12.f * uu + 15.f)) * du;
    return uu * uu * uu * poly + 1.f;
  }
  dsw = 0.f;
  return 0.f;
}

// environment of one slot (the same arithmetic as the tensor-core path)
// whose list entry nb the caller has read already
__device__ __forceinline__ void slot_env(const DescParams<float>& p, int row, int ti, int slot, int nb, SlotEnv& s) {
  const int f = p.nloc_div.div(row), i = row - f * p.nloc;
  s.nb = nb;
  const float* av = p.davg + ((size_t)ti * p.nnei + slot) * 4;
  const float* sdi = p.dstd_inv + ((size_t)ti * p.nnei + slot) * 4;
  float e4[4] = {0.f, 0.f, 0.f, 0.f};
  s.d[0] = s.d[1] = s.d[2] = 0.f;
  int keep = 1;
  if (s.nb >= 0) {
    // the displacement from the FP32 hi + lo splits (no FP64 instructions:
    // GB300's FP64 pipe is narrow)
    const int tj = pair_disp_f(p, f, i, s.nb, s.d);
    keep = p.pair_mask ? p.pair_mask[ti * p.ntypes + tj] : 1;
    if (keep) {
      const float nr2 = s.d[0] * s.d[0] + s.d[1] * s.d[1] + s.d[2] * s.d[2];
      const float nr = sqrtf(nr2);
      const float inr = 1.f / nr;
      float dsw;
      const float sw = switch_f(nr, (float)p.rcut_smth, (float)p.rcut, dsw);
      const float inr2 = inr * inr;
      e4[0] = inr * sw;
      e4[1] = s.d[0] * inr2 * sw;
      e4[2] = s.d[1] * inr2 * sw;
      e4[3] = s.d[2] * inr2 * sw;
    }
  }
#pragma unroll
  for (int c = 0; c < 4; ++c) s.rn[c] = (s.nb >= 0 && !keep) ? 0.f : (e4[c] - av[c]) * sdi[c];
  s.active = s.nb >= 0 ? keep : !p.pad_zero;
}
__device__ __forceinline__ void slot_env(const DescParams<float>& p, int row, int ti, int slot, SlotEnv& s) {
  slot_env(p, row, ti, slot, p.nlist[(size_t)row * p.nnei + slot], s);
}

// d e / d r_centre of a kept pair (source/lib/src/env_mat.cc:156-216), FP32
__device__ __forceinline__ void slot_deriv(const float d[3], float rmin, float rmax, float der[12]) {
  const float nr2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
  const float nr = sqrtf(nr2);
  const float inr = 1.f / nr;
  float dsw;
  const float sw = switch_f(nr, rmin, rmax, dsw);
  const float inr2 = inr * inr, inr3 = inr2 * inr, inr4 = inr2 * inr2;
  const float v0 = inr;
  const float v[3] = {d[0] * inr2, d[1] * inr2, d[2] * inr2};
#pragma unroll
  for (int k = 0; k < 3; ++k) der[k] = d[k] * inr3 * sw - v0 * dsw * d[k] * inr;
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int k = 0; k < 3; ++k)
      der[3 + 3 * c + k] = (2.f * d[c] * d[k] * inr4 - (c == k ? inr2 : 0.f)) * sw - v[c] * dsw * d[k] * inr;
}

// ---------------------------------------------------------------------------
// Both kernels run one CTA per SM (kFwdWarps / kBwdWarps warps) over the work chunks
// (contiguous type-sorted atoms of one centre type), section by section:
// for a section the CTA stages rows [0, rows) of that section's table in
// shared memory (the intervals of all but the closest neighbours; a pair
// in a row beyond them reads the table from global memory), then each warp
// takes one atom at a time.  Lane l owns neurons l, l + 32, l + 64, l + 96,
// so one pair's coefficients are one contiguous run of the row; a pair in
// the same interval as the previous one (neighbours come sorted by
// distance) reuses the coefficients already in registers.  The lanes
// compute the environment of 32 slots at once and park it in a per-warp
// shared-memory slot buffer, from which every lane reads each kept pair.
// Sections after the first add to the atom's xyz (forward) and virial
// (backward) where the previous section left them (the same CTA, after a
// barrier).  Sums run in a fixed order: results are bitwise reproducible.
// The forward can keep each real pair's environment (R~ and the
// displacement, two float4) for the backward, which then reads it instead
// of forming it again from the coordinates.
constexpr int kFwdWarps = 16;
constexpr int kBwdWarps = 16;
constexpr int kTabJ = 4;       // neurons per lane (ng <= 128)

struct SlotBuf {  // one kept slot, as the lanes read it (32 bytes)
  float4 rn;
  float xx, delta;
  int idx, pad;
};

// shared memory: the staged rows, then 32 slot buffers per warp
__host__ __device__ inline size_t tab_table_bytes(int rows, int ng) {
  return ((size_t)rows * 6 * ng * sizeof(float) + 15) / 16 * 16;
}

// stage rows [0, rows) of a net's table (6 ng floats a row; the table
// starts 8-byte aligned)
__device__ __forceinline__ void stage_rows(float* dst, const float* __restrict__ src, int rows, int ng) {
  const int n2 = rows * 3 * ng;  // float2 count
  const float2* s2 = reinterpret_cast<const float2*>(src);
  float2* d2 = reinterpret_cast<float2*>(dst);
  for (int q = threadIdx.x; q < n2; q += blockDim.x) d2[q] = __ldg(s2 + q);
}

// the same with a row stride of row_stride floats (even) and the neurons
// interleaved in pairs: float2 6 m + c of a staged row holds coefficient c
// of neurons 2 m and 2 m + 1 (a neuron past ng reads as zeros), so that one
// packed FMA evaluates both neurons
__device__ __forceinline__ void stage_rows_paired(float* dst, const float* __restrict__ src, int rows, int ng,
                                                  int row_stride) {
  const int per = 3 * ((ng + 1) & ~1);  // float2 per staged row
  float2* d2 = reinterpret_cast<float2*>(dst);
  const int s2stride = row_stride / 2;
  for (int q = threadIdx.x; q < rows * per; q += blockDim.x) {
    const int rr = q / per, k = q - rr * per;
    const int m = k / 6, c = k - 6 * m, n = 2 * m;
    const float* row = src + (size_t)rr * 6 * ng;
    d2[(size_t)rr * s2stride + k] = make_float2(__ldg(row + 6 * n + c), n + 1 < ng ? __ldg(row + 6 * n + 6 + c) : 0.f);
  }
}

// component c of dX[n] in the paired copy of an atom's dE/dxyz: float4
// 2 m holds (x, y) and 2 m + 1 holds (z, w) of neurons 2 m and 2 m + 1,
// each as a (neuron 2 m, neuron 2 m + 1) pair
__device__ __forceinline__ float paired_dx(const float4* s_dx, int n, int c) {
  return reinterpret_cast<const float*>(s_dx)[(n >> 1) * 8 + 2 * c + (n & 1)];
}

// the lane's coefficients of interval ix: staged rows from shared memory,
// the others from global memory
// (ix is the same in every lane: the branch does not diverge)
template <int J = kTabJ>
__device__ __forceinline__ void load_coeffs(const float* s_tab, const float* __restrict__ tab, int rows, int ix,
                                            int ng, int lane, float (&a)[kTabJ][6]) {
  auto put = [&](int j, float2 x0, float2 x1, float2 x2) {
    a[j][0] = x0.x;
    a[j][1] = x0.y;
    a[j][2] = x1.x;
    a[j][3] = x1.y;
    a[j][4] = x2.x;
    a[j][5] = x2.y;
  };
  if (ix < rows) {
    const float2* q = reinterpret_cast<const float2*>(s_tab + (size_t)ix * 6 * ng + 6 * lane);
#pragma unroll
    for (int j = 0; j < J; ++j)
      if (lane + 32 * j < ng) put(j, q[96 * j], q[96 * j + 1], q[96 * j + 2]);  // 32 neurons = 96 float2
  } else {
    const float2* q = reinterpret_cast<const float2*>(tab + (size_t)ix * 6 * ng + 6 * lane);
#pragma unroll
    for (int j = 0; j < J; ++j)
      if (lane + 32 * j < ng) put(j, __ldg(q + 96 * j), __ldg(q + 96 * j + 1), __ldg(q + 96 * j + 2));
  }
}

// The warps of a CTA take a chunk's atoms from a shared counter: warp w
// starts with atoms row0 + w and row0 + W + w, and each atom it finishes
// hands it the next one from the counter, so that it knows its next atom
// one ahead (for the prefetches) and the warps reach the section's barrier
// within about one atom of each other.  An atom's sums run in one warp in a
// fixed order, whichever warp takes it: results do not depend on the
// assignment.
__device__ __forceinline__ int take_atom(int* s_next, int& r_next, int lane) {
  int g = 0;
  if (lane == 0) g = atomicAdd(s_next, 1);
  g = __shfl_sync(0xffffffffu, g, 0);
  const int r = r_next;
  r_next = g;
  return r;
}

// TG: 0, or the lane-group size (4 or 8) of the tail neurons 32 (kTabJ - 1)
// .. ng - 1 (at most TG of them): those are not walked by the per-pair loop
// (where all 32 lanes would step through them for the few lanes that hold
// one) but afterwards, 32 / TG pairs at a time, TG lanes per pair, and
// summed across the groups at the end of the atom's section.
template <int TG>
__global__ void __launch_bounds__(kFwdWarps * 32, 1)
tab_fwd_kernel(DescParams<float> p, EmbParams<float> e, const WorkChunk* __restrict__ chunks, int nchunks,
               const int* __restrict__ sorted_rows, int rows_cap, float* __restrict__ xyz, void* __restrict__ Dout,
               int d_bf16, int* __restrict__ queue, float4* __restrict__ env_out) {
  extern __shared__ float4 smem4[];
  const int ng = p.ng, M = p.axis;
  float* s_tab = reinterpret_cast<float*>(smem4);
  SlotBuf* s_slot = reinterpret_cast<SlotBuf*>(reinterpret_cast<unsigned char*>(smem4) + tab_table_bytes(rows_cap, ng));
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  SlotBuf* my = s_slot + warp * 32;
  const float inv = 1.f / (float)p.nnei;
  const int dim = ng * M;
  __shared__ int s_work, s_next;
  for (int c = work_first(queue, &s_work); c < nchunks; c = work_next(queue, c, &s_work)) {
    const WorkChunk ch = chunks[c];
    const int ti = ch.ti;
    for (int sec = 0; sec < p.ntypes; ++sec) {
      const int net = p.type_one_side ? sec : sec * p.ntypes + ti;
      const TabMeta<float> tm = e.meta[net];
      const float* tab = e.table + tm.offset;
      const int rows = min(rows_cap, tm.hi_idx + 1);
      __syncthreads();  // the previous section's rows are no longer read
      stage_rows(s_tab, tab, rows, ng);
      if (threadIdx.x == 0) s_next = ch.row0 + 2 * kFwdWarps;
      __syncthreads();
      const bool last = sec == p.ntypes - 1;
      int r_next = ch.row0 + kFwdWarps + warp;
      for (int r = ch.row0 + warp; r < ch.row1; r = take_atom(&s_next, r_next, lane)) {
        const int row = sorted_rows[r];
        float* xr = xyz + (size_t)row * 4 * ng;
        if (r_next < ch.row1) {
          // the warp's next atom: its list section (and, after the first
          // section, its xyz so far) move into L2 while this atom is processed
          const int nrow = sorted_rows[r_next];
          const char* nlr = reinterpret_cast<const char*>(p.nlist + (size_t)nrow * p.nnei + p.sec[sec]);
          if (lane * 128 < 4 * (p.sec[sec + 1] - p.sec[sec])) prefetch_l2(nlr + lane * 128);
          if (sec > 0 && lane * 128 < 16 * ng) prefetch_l2(reinterpret_cast<const char*>(xyz + (size_t)nrow * 4 * ng) + lane * 128);
        }
        float acc[4][kTabJ];
#pragma unroll
        for (int cc = 0; cc < 4; ++cc)
#pragma unroll
          for (int j = 0; j < kTabJ; ++j) {
            const int n = lane + 32 * j;
            acc[cc][j] = (sec > 0 && n < ng) ? xr[cc * ng + n] : 0.f;
          }
        constexpr int J = TG ? kTabJ - 1 : kTabJ;  // neuron steps of the per-pair loop
        int cur = -1;
        float a[kTabJ][6] = {};  // lanes past ng keep zeros (a zero G adds nothing to the sums)
        float tacc[4] = {0.f, 0.f, 0.f, 0.f};  // the lane's tail-neuron partial sums
        const int* nlr = p.nlist + (size_t)row * p.nnei;
        int nb_next = p.sec[sec] + lane < p.sec[sec + 1] ? nlr[p.sec[sec] + lane] : -1;
        for (int base = p.sec[sec]; base < p.sec[sec + 1]; base += 32) {
          const int slot = base + lane;
          const int nb_cur = nb_next;
          nb_next = slot + 32 < p.sec[sec + 1] ? nlr[slot + 32] : -1;  // the next batch's entry, loaded ahead
          SlotEnv s;
          s.active = 0;
          if (slot < p.sec[sec + 1]) {
            slot_env(p, row, ti, slot, nb_cur, s);
            table_locate(tm, s.rn[0], s.idx, s.xx, s.delta);
            if (env_out && s.nb >= 0) {  // the pair's environment, for the backward
              float4* eo = env_out + 2 * ((size_t)row * p.nnei + slot);
              eo[0] = make_float4(s.rn[0], s.rn[1], s.rn[2], s.rn[3]);
              eo[1] = make_float4(s.d[0], s.d[1], s.d[2], s.active ? 1.f : 0.f);
            }
          }
          const unsigned m = __ballot_sync(0xffffffffu, s.active);
          if (!m) continue;
          const int cnt = __popc(m);
          if (s.active) {  // the kept slots packed in lane order
            SlotBuf b;
            b.rn = make_float4(s.rn[0], s.rn[1], s.rn[2], s.rn[3]);
            b.xx = s.xx;
            b.delta = s.delta;
            b.idx = s.idx;
            b.pad = 0;
            my[__popc(m & ((1u << lane) - 1u))] = b;
          }
          __syncwarp();
#pragma unroll 2
          for (int k = 0; k < cnt; ++k) {
            const SlotBuf b = my[k];
            if (b.idx != cur) {
              cur = b.idx;
              load_coeffs<J>(s_tab, tab, rows, cur, ng, lane, a);
            }
            float G[J];
            if (b.delta == 0.f) {  // inside the table (the same branch in every lane)
#pragma unroll
              for (int j = 0; j < J; ++j)
                G[j] = fmaf(fmaf(fmaf(fmaf(fmaf(a[j][5], b.xx, a[j][4]), b.xx, a[j][3]), b.xx, a[j][2]), b.xx,
                                 a[j][1]),
                            b.xx, a[j][0]);
            } else {  // linear extension past the ends of the table
#pragma unroll
              for (int j = 0; j < J; ++j) {
                float Gp;
                table_poly(a[j], b.xx, b.delta, G[j], Gp);
              }
            }
#pragma unroll
            for (int j = 0; j < J; ++j) {
              acc[0][j] = fmaf(b.rn.x, G[j], acc[0][j]);
              acc[1][j] = fmaf(b.rn.y, G[j], acc[1][j]);
              acc[2][j] = fmaf(b.rn.z, G[j], acc[2][j]);
              acc[3][j] = fmaf(b.rn.w, G[j], acc[3][j]);
            }
          }
          if (TG) {  // the tail neurons: lane group k % (32 / TG) takes pair k, lane q of it neuron 32 J + q
            const int q = lane % TG, n = 32 * J + q;
            if (n < ng)
              for (int k = lane / TG; k < cnt; k += 32 / (TG ? TG : 32)) {
                const SlotBuf b = my[k];
                const float2* c2 = reinterpret_cast<const float2*>(
                    (b.idx < rows ? s_tab : tab) + (size_t)b.idx * 6 * ng + 6 * n);
                float c6[6];
                float2 x0, x1, x2;
                if (b.idx < rows) {
                  x0 = c2[0];
                  x1 = c2[1];
                  x2 = c2[2];
                } else {
                  x0 = __ldg(c2);
                  x1 = __ldg(c2 + 1);
                  x2 = __ldg(c2 + 2);
                }
                c6[0] = x0.x;
                c6[1] = x0.y;
                c6[2] = x1.x;
                c6[3] = x1.y;
                c6[4] = x2.x;
                c6[5] = x2.y;
                float G, Gp;
                if (b.delta == 0.f)
                  G = fmaf(fmaf(fmaf(fmaf(fmaf(c6[5], b.xx, c6[4]), b.xx, c6[3]), b.xx, c6[2]), b.xx, c6[1]), b.xx,
                           c6[0]);
                else
                  table_poly(c6, b.xx, b.delta, G, Gp);
                tacc[0] = fmaf(b.rn.x, G, tacc[0]);
                tacc[1] = fmaf(b.rn.y, G, tacc[1]);
                tacc[2] = fmaf(b.rn.z, G, tacc[2]);
                tacc[3] = fmaf(b.rn.w, G, tacc[3]);
              }
          }
          __syncwarp();  // the slot buffer is refilled by the next 32 slots
        }
        if (TG) {  // sum the tail neurons' partials over the lane groups into lanes 0 .. TG - 1
#pragma unroll
          for (int cc = 0; cc < 4; ++cc) {
#pragma unroll
            for (int o = TG; o < 32; o <<= 1) tacc[cc] += __shfl_xor_sync(0xffffffffu, tacc[cc], o);
            if (lane < TG) acc[cc][kTabJ - 1] += tacc[cc];
          }
        }
        if (!last) {
#pragma unroll
          for (int cc = 0; cc < 4; ++cc)
#pragma unroll
            for (int j = 0; j < kTabJ; ++j) {
              const int n = lane + 32 * j;
              if (n < ng) xr[cc * ng + n] = acc[cc][j];
            }
          continue;
        }
#pragma unroll
        for (int j = 0; j < kTabJ; ++j) {
          const int n = lane + 32 * j;
#pragma unroll
          for (int cc = 0; cc < 4; ++cc) {
            acc[cc][j] *= inv;
            if (n < ng) xr[cc * ng + n] = acc[cc][j];
          }
        }
        // D[n][m] = sum_c X[c][n] X[c][m], m < M <= 32: X[c][m] sits in lane m
        if (M == 16) {  // the lane's row of D (16 values) as two or four 16-byte stores
          // X[:][m < 16] (and the tail neurons' X) through the warp's slot
          // buffer, read back as broadcasts
          float4* xs = reinterpret_cast<float4*>(my);
          __syncwarp();
          if (lane < 16) xs[lane] = make_float4(acc[0][0], acc[1][0], acc[2][0], acc[3][0]);
          if (TG && lane < TG)
            xs[16 + lane] = make_float4(acc[0][kTabJ - 1], acc[1][kTabJ - 1], acc[2][kTabJ - 1], acc[3][kTabJ - 1]);
          __syncwarp();
#pragma unroll
          for (int j = 0; j < J; ++j) {
            const int n = lane + 32 * j;
            float o[16];
#pragma unroll
            for (int mm = 0; mm < 16; ++mm) {
              const float4 x = xs[mm];
              o[mm] = fmaf(acc[3][j], x.w, fmaf(acc[2][j], x.z, fmaf(acc[1][j], x.y, acc[0][j] * x.x)));
            }
            if (n >= ng) continue;
            const size_t at = (size_t)r * dim + (size_t)n * 16;
            if (d_bf16) {
              __nv_bfloat162 h[8];
#pragma unroll
              for (int i = 0; i < 8; ++i) h[i] = __floats2bfloat162_rn(o[2 * i], o[2 * i + 1]);
              uint4* dst = reinterpret_cast<uint4*>(reinterpret_cast<__nv_bfloat16*>(Dout) + at);
              dst[0] = *reinterpret_cast<const uint4*>(&h[0]);
              dst[1] = *reinterpret_cast<const uint4*>(&h[4]);
            } else {
              float4* dst = reinterpret_cast<float4*>(reinterpret_cast<float*>(Dout) + at);
#pragma unroll
              for (int i = 0; i < 4; ++i) dst[i] = make_float4(o[4 * i], o[4 * i + 1], o[4 * i + 2], o[4 * i + 3]);
            }
          }
          if (TG) {  // the tail neurons' rows of D: lane takes neuron 32 J + lane / 8, columns 2 (lane % 8), + 1
            const int q = lane >> 3, mc = 2 * (lane & 7), n = 32 * J + q;
            if (q < TG && n < ng) {
              const float4 xn = xs[16 + q], a0 = xs[mc], a1 = xs[mc + 1];
              const float o0 = fmaf(xn.w, a0.w, fmaf(xn.z, a0.z, fmaf(xn.y, a0.y, xn.x * a0.x)));
              const float o1 = fmaf(xn.w, a1.w, fmaf(xn.z, a1.z, fmaf(xn.y, a1.y, xn.x * a1.x)));
              const size_t at = (size_t)r * dim + (size_t)n * 16 + mc;
              if (d_bf16)
                *reinterpret_cast<__nv_bfloat162*>(reinterpret_cast<__nv_bfloat16*>(Dout) + at) =
                    __floats2bfloat162_rn(o0, o1);
              else
                *reinterpret_cast<float2*>(reinterpret_cast<float*>(Dout) + at) = make_float2(o0, o1);
            }
          }
          continue;
        }
#pragma unroll
        for (int j = 0; j < kTabJ; ++j) {
          const int n = lane + 32 * j;
          for (int m0 = 0; m0 < M; m0 += 8) {
            float o[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) {
              const int mm = m0 + q;
              float sacc = 0.f;
#pragma unroll
              for (int cc = 0; cc < 4; ++cc)
                sacc = fmaf(acc[cc][j], __shfl_sync(0xffffffffu, acc[cc][0], mm & 31), sacc);
              o[q] = sacc;
            }
            if (n < ng) {
              for (int q = 0; q < 8 && m0 + q < M; ++q) {
                const size_t at = (size_t)r * dim + (size_t)n * M + m0 + q;
                if (d_bf16)
                  reinterpret_cast<__nv_bfloat16*>(Dout)[at] = __float2bfloat16_rn(o[q]);
                else
                  reinterpret_cast<float*>(Dout)[at] = o[q];
              }
            }
          }
        }
      }
    }
  }
}

// Backward: one lane per real pair.  The warp first lists the slots of the
// atom's section that hold a neighbour (in a per-warp shared list; padding
// slots get a zero gradient), then takes them 32 at a time: each lane forms
// its pair's environment and walks all neurons of its interval's staged row
// (a pair whose row is not staged is walked by the whole warp, one neuron
// per lane, after the others),
// G and G' in one Horner pass, dR~[c] += G dX[c] and P[c] += G' dX[c]
// (ds = sum_c R~[c] P[c]) with dX[n] broadcast from the warp's copy of the
// atom's dE/dxyz.  Everything is summed in the lane: no cross-lane
// reductions.  Rows are staged with an odd float2 stride, so 16 lanes on 16
// different rows read 16 different bank pairs, and with the neurons
// interleaved in pairs (as is the copy of dE/dxyz): the two neurons of a
// pair go through the packed FP32 FMA together (two IEEE fmaf results per
// instruction), even neurons into one partial sum and odd ones into another.
// KEY: kKeyAny, or the kind of list (kKeyModel, kKeyBatch, kKeyExt) when
// the pairs' environments come from the forward (env_in) and the forces go
// to the fixed-point sums (p.facc): that case is compiled without the
// other paths' branches, the neighbour's row found without run-time tests
template <int KEY>
__global__ void __launch_bounds__(kBwdWarps * 32, 1)
tab_bwd_kernel(DescParams<float> p, EmbParams<float> e, const WorkChunk* __restrict__ chunks, int nchunks,
               const int* __restrict__ sorted_rows, int rows_cap, int row_stride, const float* __restrict__ dxyz,
               float* __restrict__ gpair, double* __restrict__ vir_row, int* __restrict__ queue,
               const float4* __restrict__ env_in) {
  extern __shared__ float4 smem4[];
  const int ng = p.ng;
  float* s_tab = reinterpret_cast<float*>(smem4);
  unsigned char* tail = reinterpret_cast<unsigned char*>(smem4) + (((size_t)rows_cap * row_stride * 4 + 15) / 16 * 16);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int ng2 = (ng + 1) & ~1;                                                          // even
  float4* s_dx = reinterpret_cast<float4*>(tail) + (size_t)warp * ng2;                   // [warp][ng2], paired
  int* s_list = reinterpret_cast<int*>(reinterpret_cast<float4*>(tail) + (size_t)kBwdWarps * ng2) +
                (size_t)warp * p.nnei;                                                     // [warp][nnei]
  int* s_perm = reinterpret_cast<int*>(reinterpret_cast<float4*>(tail) + (size_t)kBwdWarps * ng2) +
                (size_t)kBwdWarps * p.nnei + warp * 32;                                    // [warp][32]
  const float rmin = (float)p.rcut_smth, rmax = (float)p.rcut;
  const int bank_step = (row_stride / 2) & 15;  // a row's 8-byte bank pair advances by this per row
  __shared__ int s_work, s_next;
  for (int c = work_first(queue, &s_work); c < nchunks; c = work_next(queue, c, &s_work)) {
    const WorkChunk ch = chunks[c];
    const int ti = ch.ti;
    for (int sec = 0; sec < p.ntypes; ++sec) {
      const int net = p.type_one_side ? sec : sec * p.ntypes + ti;
      const TabMeta<float> tm = e.meta[net];
      const float* tab = e.table + tm.offset;
      const int rows = min(rows_cap, tm.hi_idx + 1);
      __syncthreads();
      stage_rows_paired(s_tab, tab, rows, ng, row_stride);
      if (threadIdx.x == 0) s_next = ch.row0 + 2 * kBwdWarps;
      __syncthreads();
      int r_next = ch.row0 + kBwdWarps + warp;
      for (int r = ch.row0 + warp; r < ch.row1; r = take_atom(&s_next, r_next, lane)) {
        const int row = sorted_rows[r];
        const int* nl = p.nlist + (size_t)row * p.nnei;
        float* gp_row = gpair + (size_t)row * p.nnei * 3;
        if (r_next < ch.row1) {
          // the warp's next atom: its dE/dxyz, list and first pair
          // environments move into L2 while this atom is processed
          const int nrow = sorted_rows[r_next];
          const char* nd = reinterpret_cast<const char*>(dxyz + (size_t)nrow * 4 * ng);
          if (lane * 128 < 16 * ng) prefetch_l2(nd + lane * 128);
          if (lane * 128 < 4 * p.nnei) prefetch_l2(reinterpret_cast<const char*>(p.nlist + (size_t)nrow * p.nnei) + lane * 128);
          if (env_in && p.sec[sec] + lane < p.sec[sec + 1])
            prefetch_l2(env_in + 2 * ((size_t)nrow * p.nnei + p.sec[sec] + lane));
        }
        // the atom's dE/dxyz (dxyz is [row][ng][4]), paired, and the section's real slots
        for (int m = lane; 2 * m < ng; m += 32) {
          const float4* src = reinterpret_cast<const float4*>(dxyz + (size_t)row * 4 * ng) + 2 * m;
          const float4 a = src[0], b = 2 * m + 1 < ng ? src[1] : make_float4(0.f, 0.f, 0.f, 0.f);
          s_dx[2 * m] = make_float4(a.x, b.x, a.y, b.y);
          s_dx[2 * m + 1] = make_float4(a.z, b.z, a.w, b.w);
        }
        int nreal = 0;
        for (int base = p.sec[sec]; base < p.sec[sec + 1]; base += 32) {
          const int slot = base + lane;
          const bool have = slot < p.sec[sec + 1];
          const bool real = have && nl[slot] >= 0;
          const unsigned m = __ballot_sync(0xffffffffu, real);
          if (real) s_list[nreal + __popc(m & ((1u << lane) - 1u))] = slot;
          if (have && !real && !(KEY != kKeyAny || p.facc)) {
            gp_row[3 * slot] = 0.f;
            gp_row[3 * slot + 1] = 0.f;
            gp_row[3 * slot + 2] = 0.f;
          }
          nreal += __popc(m);
        }
        __syncwarp();
        float vir_hi[9], vir_lo[9];  // compensated FP32 sums of the lane's pairs
#pragma unroll
        for (int k = 0; k < 9; ++k) vir_hi[k] = vir_lo[k] = 0.f;
        float own[3] = {0.f, 0.f, 0.f};  // fixed-point forces: the row's share of the lane's pairs
        for (int q0 = 0; q0 < nreal; q0 += 32) {
          const bool mine = q0 + lane < nreal;
          const int slot = mine ? s_list[q0 + lane] : p.sec[sec];
          if (env_in && q0 + 32 + lane < nreal)  // the next 32 pairs' environments
            prefetch_l2(env_in + 2 * ((size_t)row * p.nnei + s_list[q0 + 32 + lane]));
          SlotEnv s;
          s.active = 0;
          if (mine) {
            if (KEY != kKeyAny || env_in) {  // the environment the forward formed for this pair
              const float4* ei = env_in + 2 * ((size_t)row * p.nnei + slot);
              const float4 a = __ldg(ei), b = __ldg(ei + 1);
              s.nb = 0;
              s.rn[0] = a.x;
              s.rn[1] = a.y;
              s.rn[2] = a.z;
              s.rn[3] = a.w;
              s.d[0] = b.x;
              s.d[1] = b.y;
              s.d[2] = b.z;
              s.active = b.w != 0.f;
            } else {
              slot_env(p, row, ti, slot, s);
            }
            table_locate(tm, s.rn[0], s.idx, s.xx, s.delta);
          }
          bool act = mine && s.active;  // excluded type pairs carry no gradient
          int slot_p = slot;
          bool mine_p = mine;
          {
            // Lanes for the pairs such that each half-warp's 8-byte
            // coefficient loads spread over the 16 bank pairs: the distinct
            // staged rows of one bank class (row * bank_step mod 16) go to
            // the two halves in turn (a row's repeats stay with it, a
            // broadcast); pairs with no staged row fill the free lanes.
            const unsigned full = 0xffffffffu, lt = (1u << lane) - 1u;
            const bool has = act && s.idx < rows && s.delta == 0.f;
            const int cls = (s.idx * bank_step) & 15;
            const unsigned m_row = __match_any_sync(full, has ? s.idx : -1 - lane);
            const int first = __ffs(m_row) - 1;
            const unsigned firsts = __ballot_sync(full, has && lane == first);
            const unsigned m_cls = __match_any_sync(full, has ? cls : -64 - lane);
            const int half = has ? (__popc(m_cls & firsts & ((1u << first) - 1u)) & 1) : 2;
            const unsigned A = __ballot_sync(full, half == 0), B = __ballot_sync(full, half == 1),
                           F = __ballot_sync(full, half == 2);
            const int nA = __popc(A), nB = __popc(B);
            const int a_keep = min(nA, 16), b_keep = min(nB, 16);
            const int a_occ = a_keep + max(nB - 16, 0), b_occ = b_keep + max(nA - 16, 0);
            int pos;
            if (half == 0) {
              const int k = __popc(A & lt);
              pos = k < 16 ? k : 16 + b_keep + (k - 16);
            } else if (half == 1) {
              const int k = __popc(B & lt);
              pos = k < 16 ? 16 + k : a_keep + (k - 16);
            } else {
              const int k = __popc(F & lt);
              pos = k < 16 - a_occ ? a_occ + k : 16 + b_occ + (k - (16 - a_occ));
            }
            s_perm[pos] = lane;
            __syncwarp();
            const int src = s_perm[lane];
            __syncwarp();  // read before the next batch writes
#pragma unroll
            for (int c = 0; c < 4; ++c) s.rn[c] = __shfl_sync(full, s.rn[c], src);
#pragma unroll
            for (int c = 0; c < 3; ++c) s.d[c] = __shfl_sync(full, s.d[c], src);
            s.idx = __shfl_sync(full, s.idx, src);
            s.xx = __shfl_sync(full, s.xx, src);
            s.delta = __shfl_sync(full, s.delta, src);
            slot_p = __shfl_sync(full, slot, src);
            act = __shfl_sync(full, (int)act, src) != 0;
            mine_p = __shfl_sync(full, (int)mine, src) != 0;
          }
          // a pair whose interval's row is not staged (the closest
          // neighbours), or that lies past the ends of the table (linear
          // extension), is walked by the whole warp below, so that the
          // lane-per-pair loop reads shared memory only and evaluates the
          // plain quintic
          const bool glob = act && (s.idx >= rows || s.delta != 0.f);
          float dR[4] = {0.f, 0.f, 0.f, 0.f}, Pc[4] = {0.f, 0.f, 0.f, 0.f};
          if (act && !glob) {
            const float2* rowc = reinterpret_cast<const float2*>(s_tab + (size_t)s.idx * row_stride);
            const float2 xx = make_float2(s.xx, s.xx);
            // neurons 2 m (.x) and 2 m + 1 (.y) per step, even and odd
            // neurons into their own partial sums, added at the end
            float2 r2[4], pc2[4];
#pragma unroll
            for (int cc = 0; cc < 4; ++cc) r2[cc] = pc2[cc] = make_float2(0.f, 0.f);
#pragma unroll 10
            for (int m = 0; 2 * m < ng; ++m) {
              const float2* q = rowc + 6 * m;  // coefficient c of both neurons
              const float2 c0 = q[0], c1 = q[1], c2 = q[2], c3 = q[3], c4 = q[4], c5 = q[5];
              const float4 dxy = s_dx[2 * m], dzw = s_dx[2 * m + 1];
              // value and derivative of the quintic in one Horner pass
              float2 G = __ffma2_rn(c5, xx, c4), Gp = c5;
              Gp = __ffma2_rn(Gp, xx, G);
              G = __ffma2_rn(G, xx, c3);
              Gp = __ffma2_rn(Gp, xx, G);
              G = __ffma2_rn(G, xx, c2);
              Gp = __ffma2_rn(Gp, xx, G);
              G = __ffma2_rn(G, xx, c1);
              Gp = __ffma2_rn(Gp, xx, G);
              G = __ffma2_rn(G, xx, c0);
              const float2 d[4] = {make_float2(dxy.x, dxy.y), make_float2(dxy.z, dxy.w), make_float2(dzw.x, dzw.y),
                                   make_float2(dzw.z, dzw.w)};
#pragma unroll
              for (int cc = 0; cc < 4; ++cc) {
                r2[cc] = __ffma2_rn(G, d[cc], r2[cc]);
                pc2[cc] = __ffma2_rn(Gp, d[cc], pc2[cc]);
              }
            }
#pragma unroll
            for (int cc = 0; cc < 4; ++cc) {
              dR[cc] = r2[cc].x + r2[cc].y;
              Pc[cc] = pc2[cc].x + pc2[cc].y;
            }
          }
          // rows in global memory: lane l takes neurons l, l + 32, ... of
          // the pair's row (coalesced reads), then fixed-order warp sums
          unsigned gm = __ballot_sync(0xffffffffu, glob);
          while (gm) {
            const int src = __ffs(gm) - 1;
            gm &= gm - 1;
            const int gi = __shfl_sync(0xffffffffu, s.idx, src);
            const float gx = __shfl_sync(0xffffffffu, s.xx, src), gd = __shfl_sync(0xffffffffu, s.delta, src);
            const float2* grow = reinterpret_cast<const float2*>(tab + (size_t)gi * 6 * ng);
            float r[4] = {0.f, 0.f, 0.f, 0.f}, pc[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (int j = 0; j < kTabJ; ++j) {
              const int n = lane + 32 * j;
              if (n < ng) {
                const float2 x0 = __ldg(grow + 3 * n), x1 = __ldg(grow + 3 * n + 1), x2 = __ldg(grow + 3 * n + 2);
                const float4 d = make_float4(paired_dx(s_dx, n, 0), paired_dx(s_dx, n, 1), paired_dx(s_dx, n, 2),
                                             paired_dx(s_dx, n, 3));
                float G = fmaf(x2.y, gx, x2.x), Gp = x2.y;
                Gp = fmaf(Gp, gx, G);
                G = fmaf(G, gx, x1.y);
                Gp = fmaf(Gp, gx, G);
                G = fmaf(G, gx, x1.x);
                Gp = fmaf(Gp, gx, G);
                G = fmaf(G, gx, x0.y);
                Gp = fmaf(Gp, gx, G);
                G = fmaf(G, gx, x0.x);
                G = fmaf(Gp, gd, G);
                r[0] = fmaf(G, d.x, r[0]);
                r[1] = fmaf(G, d.y, r[1]);
                r[2] = fmaf(G, d.z, r[2]);
                r[3] = fmaf(G, d.w, r[3]);
                pc[0] = fmaf(Gp, d.x, pc[0]);
                pc[1] = fmaf(Gp, d.y, pc[1]);
                pc[2] = fmaf(Gp, d.z, pc[2]);
                pc[3] = fmaf(Gp, d.w, pc[3]);
              }
            }
#pragma unroll
            for (int cc = 0; cc < 4; ++cc) {
              r[cc] = warp_sum(r[cc]);
              pc[cc] = warp_sum(pc[cc]);
            }
            if (lane == src) {
#pragma unroll
              for (int cc = 0; cc < 4; ++cc) {
                dR[cc] = r[cc];
                Pc[cc] = pc[cc];
              }
            }
          }
          if (mine_p) {
            float g[3] = {0.f, 0.f, 0.f};
            if (act) {
              // dR~ (+ ds through s = R~[0]) -> the pair gradient and virial
              const float ds = s.rn[0] * Pc[0] + s.rn[1] * Pc[1] + s.rn[2] * Pc[2] + s.rn[3] * Pc[3];
              dR[0] += ds;
              float der[12];
              slot_deriv(s.d, rmin, rmax, der);
              const float* sdi = p.dstd_inv + ((size_t)ti * p.nnei + slot_p) * 4;
#pragma unroll
              for (int cc = 0; cc < 4; ++cc) {
                const float w = dR[cc] * sdi[cc];
#pragma unroll
                for (int k = 0; k < 3; ++k) g[k] -= w * der[3 * cc + k];
              }
#pragma unroll
              for (int k = 0; k < 3; ++k)
#pragma unroll
                for (int l = 0; l < 3; ++l) comp_add(vir_hi[3 * k + l], vir_lo[3 * k + l], -g[k] * s.d[l]);
            }
            if (KEY != kKeyAny || p.facc) {
              if (act) {  // -g onto the neighbour's row
                unsigned long long* a = p.facc + 3 * (size_t)neighbour_row<KEY == kKeyAny ? kKeyAny : KEY>(p, row, nl[slot_p]);
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                  own[k] += g[k];
                  atomicAdd(a + k, (unsigned long long)__float2ll_rn(-g[k] * kFixScale));
                }
              }
            } else {
              gp_row[3 * slot_p] = g[0];
              gp_row[3 * slot_p + 1] = g[1];
              gp_row[3 * slot_p + 2] = g[2];
            }
          }
        }
        if (KEY != kKeyAny || p.facc) {
#pragma unroll
          for (int k = 0; k < 3; ++k) own[k] = warp_sum(own[k]);
          if (lane == 0)
#pragma unroll
            for (int k = 0; k < 3; ++k)
              atomicAdd(p.facc + 3 * (size_t)row + k, (unsigned long long)__float2ll_rn(own[k] * kFixScale));
        }
#pragma unroll
        for (int k = 0; k < 9; ++k) {
          const double vv = warp_comp_sum(vir_hi[k], vir_lo[k]);
          if (lane == 0) vir_row[(size_t)row * 9 + k] += vv;  // zeroed before the launch
        }
        __syncwarp();  // the warp's dX copy and slot list are reused by its next atom
      }
    }
  }
}

}  // namespace

int tab_fused_eligible(int ng, int axis) { return ng >= 1 && ng <= 32 * kTabJ && axis >= 1 && axis <= 32; }

namespace {

// staged rows: as many as fit next to the slot buffers in the opt-in maximum
int tab_rows_cap(int ng, int warps, size_t* smem) {
  int dev = 0, optin = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  const size_t slot = (size_t)warps * 32 * sizeof(SlotBuf);
  const size_t avail = (size_t)optin > slot + 1024 ? (size_t)optin - slot - 1024 : 0;
  const int rows = (int)(avail / ((size_t)6 * ng * sizeof(float)));
  *smem = tab_table_bytes(rows, ng) + slot;
  return rows;
}

}  // namespace

int launch_tab_fwd(const DescParams<float>& p, const EmbParams<float>& e, const WorkChunk* chunks, int nchunks,
                   const int* sorted_rows, float* xyz, void* D, int d_bf16, cudaStream_t st, int* queue,
                   float4* env_out) {
  if (nchunks <= 0) return DPGB_OK;
  size_t smem = 0;
  const int rows = tab_rows_cap(p.ng, kFwdWarps, &smem);
  // the neurons past the last full 32 go to the tail pass when there are at
  // most 8 of them
  const int tail = p.ng - 32 * (kTabJ - 1);
  auto run = [&](auto kern) -> int {
    DPGB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kern<<<std::min(nchunks, sm_count()), kFwdWarps * 32, smem, st>>>(p, e, chunks, nchunks, sorted_rows, rows, xyz,
                                                                        D, d_bf16, queue, env_out);
    return DPGB_OK;
  };
  if (tail >= 1 && tail <= 4)
    DPGB_TRY(run(tab_fwd_kernel<4>));
  else if (tail >= 5 && tail <= 8)
    DPGB_TRY(run(tab_fwd_kernel<8>));
  else
    DPGB_TRY(run(tab_fwd_kernel<0>));
  return check_launch("tab_fwd");
}

int launch_tab_bwd(const DescParams<float>& p, const EmbParams<float>& e, const WorkChunk* chunks, int nchunks,
                   const int* sorted_rows, const float* dxyz, float* gpair, double* vir_row, cudaStream_t st,
                   int* queue, const float4* env_in) {
  if (nchunks <= 0) return DPGB_OK;
  // rows (neurons paired, ng rounded up to even) at an odd float2 stride;
  // per warp the atom's dE/dxyz (paired) and its slot list
  const int ng2 = (p.ng + 1) & ~1;
  int per2 = 3 * ng2;
  if (per2 % 2 == 0) ++per2;
  const int row_stride = 2 * per2;
  int dev = 0, optin = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  const size_t per_warp = (size_t)ng2 * sizeof(float4) + (size_t)p.nnei * sizeof(int) + 32 * sizeof(int);
  const size_t fixed = (size_t)kBwdWarps * per_warp + 16 + 1024;
  if ((size_t)optin <= fixed) return fail(DPGB_EINVAL, "tab_bwd: the neighbour list is too wide");
  const int rows = (int)(((size_t)optin - fixed) / ((size_t)row_stride * sizeof(float)));
  const size_t smem = ((size_t)rows * row_stride * 4 + 15) / 16 * 16 + (size_t)kBwdWarps * per_warp;
  auto run = [&](auto kern) -> int {
    DPGB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kern<<<std::min(nchunks, sm_count()), kBwdWarps * 32, smem, st>>>(p, e, chunks, nchunks, sorted_rows, rows,
                                                                        row_stride, dxyz, gpair, vir_row, queue,
                                                                        env_in);
    return DPGB_OK;
  };
  const int kind = list_key_kind(p);
  if (!env_in || !p.facc)
    DPGB_TRY(run(tab_bwd_kernel<kKeyAny>));
  else if (kind == kKeyExt)
    DPGB_TRY(run(tab_bwd_kernel<kKeyExt>));
  else if (kind == kKeyBatch)
    DPGB_TRY(run(tab_bwd_kernel<kKeyBatch>));
  else
    DPGB_TRY(run(tab_bwd_kernel<kKeyModel>));
  return check_launch("tab_bwd");
}

}  // namespace dpgb
