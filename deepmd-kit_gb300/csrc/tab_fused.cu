// Compressed se_e2_a descriptor for the mixed-precision DeepPot: the table
// lookup of tabulate_fusion_se_a (source/lib/src/gpu/tabulate.cu:293-506)
// fused with the environment matrix, the G^T R~ contraction, D, and on the
// way back the pair gradients and per-atom virial — on the CUDA cores in FP32
// (the table is a per-interval quintic: no GEMM to give the tensor cores).
//
// One warp per atom (rows in type-sorted order, so the warps of a CTA share
// nets and table rows stay in L1).  Lane l owns neurons l, l+32, l+64, l+96:
// a pair's table row (6 coefficients per neuron) is read as three float2
// loads per neuron, contiguous across the warp.  The warp evaluates the
// environment of 32 slots at once (one per lane) and then walks the kept
// slots, broadcasting each slot's R~ and table interval by shuffles.
// Backward: per pair dG_n = R~ . dxyz[:, n], dR~ = sum_n G_n dxyz[:, n] plus
// ds = sum_n dG_n G'_n, reduced across the warp; the slot's owner lane turns
// dR~ into the pair gradient and the pair virial.  Sums run in a fixed order:
// results are bitwise reproducible.
#include <cuda_bf16.h>

#include "se_a.cuh"

namespace dpgb {
namespace {

constexpr int kTabWarps = 8;
constexpr int kTabJ = 4;  // neurons per lane (ng <= 128)

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
__device__ __forceinline__ void slot_env(const DescParams<float>& p, int row, int ti, int slot, SlotEnv& s) {
  const int f = p.nloc_div.div(row), i = row - f * p.nloc;
  s.nb = p.nlist[(size_t)row * p.nnei + slot];
  const float* av = p.davg + ((size_t)ti * p.nnei + slot) * 4;
  const float* sdi = p.dstd_inv + ((size_t)ti * p.nnei + slot) * 4;
  float e4[4] = {0.f, 0.f, 0.f, 0.f};
  s.d[0] = s.d[1] = s.d[2] = 0.f;
  int keep = 1;
  if (s.nb >= 0) {
    // FP64 displacement: these kernels are bound by the table reads, which
    // the split coordinates' extra loads would add to
    double dd[3];
    const int tj = pair_disp(p, f, i, s.nb, dd);
    s.d[0] = (float)dd[0];
    s.d[1] = (float)dd[1];
    s.d[2] = (float)dd[2];
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

__device__ __forceinline__ void coeffs(const float* __restrict__ rowc, float a[6]) {
  const float2* q = reinterpret_cast<const float2*>(rowc);
  const float2 x0 = __ldg(q), x1 = __ldg(q + 1), x2 = __ldg(q + 2);
  a[0] = x0.x;
  a[1] = x0.y;
  a[2] = x1.x;
  a[3] = x1.y;
  a[4] = x2.x;
  a[5] = x2.y;
}

__global__ void __launch_bounds__(kTabWarps * 32, 4)  // 4 CTAs (32 warps) per SM: the table reads want the warps
tab_fwd_kernel(DescParams<float> p, EmbParams<float> e, const int* __restrict__ sorted_rows, int nsorted,
               float* __restrict__ xyz, void* __restrict__ Dout, int d_bf16) {
  const int lane = threadIdx.x & 31;
  const int r = blockIdx.x * kTabWarps + (threadIdx.x >> 5);
  if (r >= nsorted) return;
  const int row = sorted_rows[r];
  const int ti = p.atype[row - p.nloc_div.div(row) * p.nloc];
  const int ng = p.ng, M = p.axis;
  float acc[4][kTabJ];
#pragma unroll
  for (int c = 0; c < 4; ++c)
#pragma unroll
    for (int j = 0; j < kTabJ; ++j) acc[c][j] = 0.f;
  for (int sec = 0; sec < p.ntypes; ++sec) {
    const int net = p.type_one_side ? sec : sec * p.ntypes + ti;
    const TabMeta<float> tm = e.meta[net];
    const float* tab = e.table + tm.offset;
    for (int base = p.sec[sec]; base < p.sec[sec + 1]; base += 32) {
      const int slot = base + lane;
      SlotEnv s;
      s.active = 0;
      if (slot < p.sec[sec + 1]) {
        slot_env(p, row, ti, slot, s);
        table_locate(tm, s.rn[0], s.idx, s.xx, s.delta);
      }
      unsigned m = __ballot_sync(0xffffffffu, s.active);
      while (m) {
        const int src = __ffs(m) - 1;
        m &= m - 1;
        float rr[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) rr[c] = __shfl_sync(0xffffffffu, s.rn[c], src);
        const int ix = __shfl_sync(0xffffffffu, s.idx, src);
        const float xx = __shfl_sync(0xffffffffu, s.xx, src);
        const float dl = __shfl_sync(0xffffffffu, s.delta, src);
        const float* rowc = tab + (size_t)ix * 6 * ng;
#pragma unroll
        for (int j = 0; j < kTabJ; ++j) {
          const int n = lane + 32 * j;
          if (n < ng) {
            float a[6], G, Gp;
            coeffs(rowc + 6 * n, a);
            table_poly(a, xx, dl, G, Gp);
#pragma unroll
            for (int c = 0; c < 4; ++c) acc[c][j] = fmaf(rr[c], G, acc[c][j]);
          }
        }
      }
    }
  }
  const float inv = 1.f / (float)p.nnei;
  float* xr = xyz + (size_t)row * 4 * ng;
#pragma unroll
  for (int j = 0; j < kTabJ; ++j) {
    const int n = lane + 32 * j;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      acc[c][j] *= inv;
      if (n < ng) xr[c * ng + n] = acc[c][j];
    }
  }
  // D[n][m] = sum_c X[c][n] X[c][m], m < M <= 32: X[c][m] sits in lane m
  const int dim = ng * M;
#pragma unroll
  for (int j = 0; j < kTabJ; ++j) {
    const int n = lane + 32 * j;
    for (int m0 = 0; m0 < M; m0 += 8) {
      float o[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int m = m0 + q;
        float s = 0.f;
#pragma unroll
        for (int c = 0; c < 4; ++c) s = fmaf(acc[c][j], __shfl_sync(0xffffffffu, acc[c][0], m & 31), s);
        o[q] = s;
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

__global__ void __launch_bounds__(kTabWarps * 32, 3)  // 3 CTAs (24 warps) per SM
tab_bwd_kernel(DescParams<float> p, EmbParams<float> e, const int* __restrict__ sorted_rows, int nsorted,
               const float* __restrict__ dxyz, float* __restrict__ gpair, double* __restrict__ vir_row) {
  const int lane = threadIdx.x & 31;
  const int r = blockIdx.x * kTabWarps + (threadIdx.x >> 5);
  if (r >= nsorted) return;
  const int row = sorted_rows[r];
  const int ti = p.atype[row - p.nloc_div.div(row) * p.nloc];
  const int ng = p.ng;
  const float rmin = (float)p.rcut_smth, rmax = (float)p.rcut;
  // the atom's dE/dxyz, one float4 (four components) per neuron, shared by
  // the warp's lanes (each lane walks all neurons of its own pair)
  __shared__ float4 s_dx[kTabWarps][32 * kTabJ];
  float4* sdx = s_dx[threadIdx.x >> 5];
  const float* dr = dxyz + (size_t)row * 4 * ng;
  for (int n = lane; n < ng; n += 32) sdx[n] = reinterpret_cast<const float4*>(dr)[n];  // dxyz is [row][ng][4]
  __syncwarp();
  float vir_hi[9], vir_lo[9];  // compensated FP32 sums
#pragma unroll
  for (int k = 0; k < 9; ++k) vir_hi[k] = vir_lo[k] = 0.f;
  float* gp_row = gpair + (size_t)row * p.nnei * 3;
  for (int sec = 0; sec < p.ntypes; ++sec) {
    const int net = p.type_one_side ? sec : sec * p.ntypes + ti;
    const TabMeta<float> tm = e.meta[net];
    const float* tab = e.table + tm.offset;
    for (int base = p.sec[sec]; base < p.sec[sec + 1]; base += 32) {
      const int slot = base + lane;
      SlotEnv s;
      s.active = 0;
      s.nb = -1;
      const bool have = slot < p.sec[sec + 1];
      if (have) {
        slot_env(p, row, ti, slot, s);
        table_locate(tm, s.rn[0], s.idx, s.xx, s.delta);
      }
      const bool real = have && s.nb >= 0 && s.active;  // only real kept pairs carry a gradient
      // dR~ of this lane's pair: sum over neurons of G dX (direct term) and
      // of (R~ . dX) G' (through s = R~[0]), in neuron order
      float mine[4] = {0.f, 0.f, 0.f, 0.f};
      if (real) {
        const float* rowc = tab + (size_t)s.idx * 6 * ng;
        float ds = 0.f;
        for (int n = 0; n < ng; ++n) {
          float a[6], G, Gp;
          coeffs(rowc + 6 * n, a);
          table_poly(a, s.xx, s.delta, G, Gp);
          const float4 d = sdx[n];
          const float dG = fmaf(s.rn[3], d.w, fmaf(s.rn[2], d.z, fmaf(s.rn[1], d.y, s.rn[0] * d.x)));
          mine[0] = fmaf(G, d.x, mine[0]);
          mine[1] = fmaf(G, d.y, mine[1]);
          mine[2] = fmaf(G, d.z, mine[2]);
          mine[3] = fmaf(G, d.w, mine[3]);
          ds = fmaf(dG, Gp, ds);
        }
        mine[0] += ds;
      }
      if (have) {
        float g[3] = {0.f, 0.f, 0.f};
        if (real) {
          float der[12];
          slot_deriv(s.d, rmin, rmax, der);
          const float* sdi = p.dstd_inv + ((size_t)ti * p.nnei + slot) * 4;
#pragma unroll
          for (int c = 0; c < 4; ++c) {
            const float w = mine[c] * sdi[c];
#pragma unroll
            for (int k = 0; k < 3; ++k) g[k] -= w * der[3 * c + k];
          }
#pragma unroll
          for (int k = 0; k < 3; ++k)
#pragma unroll
            for (int l = 0; l < 3; ++l) comp_add(vir_hi[3 * k + l], vir_lo[3 * k + l], -g[k] * s.d[l]);
        }
        gp_row[3 * slot] = g[0];
        gp_row[3 * slot + 1] = g[1];
        gp_row[3 * slot + 2] = g[2];
      }
    }
  }
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    const double v = warp_comp_sum(vir_hi[k], vir_lo[k]);
    if (lane == 0) vir_row[(size_t)row * 9 + k] = v;
  }
}

}  // namespace

int tab_fused_eligible(int ng, int axis) { return ng >= 1 && ng <= 32 * kTabJ && axis >= 1 && axis <= 32; }

int launch_tab_fwd(const DescParams<float>& p, const EmbParams<float>& e, const int* sorted_rows, int nsorted,
                   float* xyz, void* D, int d_bf16, cudaStream_t st) {
  if (nsorted <= 0) return DPGB_OK;
  tab_fwd_kernel<<<ceil_div(nsorted, kTabWarps), kTabWarps * 32, 0, st>>>(p, e, sorted_rows, nsorted, xyz, D, d_bf16);
  return check_launch("tab_fwd");
}

int launch_tab_bwd(const DescParams<float>& p, const EmbParams<float>& e, const int* sorted_rows, int nsorted,
                   const float* dxyz, float* gpair, double* vir_row, cudaStream_t st) {
  if (nsorted <= 0) return DPGB_OK;
  tab_bwd_kernel<<<ceil_div(nsorted, kTabWarps), kTabWarps * 32, 0, st>>>(p, e, sorted_rows, nsorted, dxyz, gpair,
                                                                          vir_row);
  return check_launch("tab_bwd");
}

}  // namespace dpgb
