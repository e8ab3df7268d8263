// Fused se_e2_a descriptor kernels (SIMT form, FP64 or FP32 arithmetic).
//
// desc_fwd: per centre atom, the environment matrix of every slot
//   (deepmd/pt/model/descriptor/env_mat.py:18-119), the embedding net of each
//   active slot (or its compressed table), xyz = sum_j R~_j^T G_j / nnei and
//   D = xyz^T xyz[:, :axis]  (se_a.py:742-858).
// desc_bwd: per centre atom, dE/dxyz from dE/dD, the embedding recomputed
//   (activations are not stored) and back-propagated to dE/dR~, then the
//   pair gradient g_ij = dE/d(r_j - r_i) and the centre-side virial.
// One CTA of 128 threads per atom; slots of a type section are processed in
// chunks of CH through shared memory.
#include <cmath>

#include "se_a.cuh"

namespace dpgb {
namespace {

constexpr int kThreads = 128;
constexpr int kMaxW = 128;    // widest embedding layer supported here
constexpr int kNQ = 4;        // 4*ng / kThreads, ng <= 128

template <typename T>
__device__ __forceinline__ T tanh_t(T x);
template <>
__device__ __forceinline__ double tanh_t<double>(double x) { return tanh(x); }
template <>
__device__ __forceinline__ float tanh_t<float>(float x) { return tanhf(x); }

template <typename T>
__device__ __forceinline__ T sqrt_t(T x);
template <>
__device__ __forceinline__ double sqrt_t<double>(double x) { return sqrt(x); }
template <>
__device__ __forceinline__ float sqrt_t<float>(float x) { return sqrtf(x); }

// R~ = s(r)[1/r, x/r^2, y/r^2, z/r^2] and (optionally) its derivative with
// respect to the centre atom, der[c*3+k]  (env_mat.cc:156-216 formulas)
template <typename T, bool DER>
__device__ __forceinline__ void env_row(const T d[3], T rmin, T rmax, T em[4], T der[12]) {
  const T nr2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
  const T nr = sqrt_t<T>(nr2);
  const T inr = (T)1 / nr;
  T sw, dsw;
  if (nr < rmin) {
    sw = (T)1;
    dsw = (T)0;
  } else if (nr < rmax) {
    const T du = (T)1 / (rmax - rmin);
    const T uu = (nr - rmin) * du;
    const T poly = (T)-6 * uu * uu + (T)15 * uu - (T)10;
    sw = uu * uu * uu * poly + (T)1;
    dsw = ((T)3 * uu * uu * poly + uu * uu * uu * ((T)-12 * uu + (T)15)) * du;
  } else {
    sw = (T)0;
    dsw = (T)0;
  }
  const T inr2 = inr * inr;
  const T v0 = inr;
  const T v[3] = {d[0] * inr2, d[1] * inr2, d[2] * inr2};
  em[0] = v0 * sw;
  em[1] = v[0] * sw;
  em[2] = v[1] * sw;
  em[3] = v[2] * sw;
  if (DER) {
    const T inr3 = inr2 * inr;
    const T inr4 = inr2 * inr2;
#pragma unroll
    for (int k = 0; k < 3; ++k) der[k] = d[k] * inr3 * sw - v0 * dsw * d[k] * inr;
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int k = 0; k < 3; ++k)
        der[3 + 3 * c + k] = ((T)2 * d[c] * d[k] * inr4 - (c == k ? inr2 : (T)0)) * sw -
                             v[c] * dsw * d[k] * inr;
  }
}

template <typename T>
struct SmemLayout {
  size_t rn, act, list, secpos, dvec, drn, xyz, dxyz, xin, buf, total;
};

template <typename T>
__host__ __device__ inline size_t align16(size_t x) {
  return (x + 15) & ~(size_t)15;
}

// shared memory layout shared by both kernels
template <typename T, int CH, bool BWD>
__host__ __device__ inline SmemLayout<T> make_layout(int nnei, int ng, int n_layer, const int* width) {
  SmemLayout<T> L;
  size_t o = 0;
  L.rn = o;     o = align16<T>(o + sizeof(T) * 4 * nnei);
  L.act = o;    o = align16<T>(o + sizeof(int) * nnei);
  L.list = o;   o = align16<T>(o + sizeof(int) * nnei);
  L.secpos = o; o = align16<T>(o + sizeof(int) * (DPGB_MAX_TYPES + 1));
  L.dvec = o;   o = align16<T>(o + (BWD ? sizeof(double) * 3 * nnei : 0));
  L.drn = o;    o = align16<T>(o + (BWD ? sizeof(T) * 4 * nnei : 0));
  L.xyz = o;    o = align16<T>(o + sizeof(T) * 4 * ng);
  L.dxyz = o;   o = align16<T>(o + (BWD ? sizeof(T) * 4 * ng : 0));
  L.xin = o;    o = align16<T>(o + sizeof(T) * CH);
  L.buf = o;
  size_t nb = 0;
  if (BWD) {
    for (int l = 0; l < n_layer; ++l) nb += 2 * (size_t)width[l];  // Y_l and T_l
    nb += 3 * (size_t)kMaxW;                                       // dY, dP, dX
  } else {
    nb = 2 * (size_t)kMaxW;
  }
  o = align16<T>(o + sizeof(T) * CH * nb);
  L.total = o;
  return L;
}

// environment of every slot of one row; returns via shared memory:
// Rn[j][4], act[j] (1 when the slot goes through the embedding), and for
// the backward pass the FP64 displacement.
template <typename T, bool BWD>
__device__ void row_env(const DescParams<T>& p, int row, int f, int i, int ti, T* s_rn, int* s_act,
                        double* s_d) {
  const T rmin = (T)p.rcut_smth, rmax = (T)p.rcut;
  for (int j = threadIdx.x; j < p.nnei; j += blockDim.x) {
    const int nb = p.nlist[(size_t)row * p.nnei + j];
    const T* av = p.davg + ((size_t)ti * p.nnei + j) * 4;
    const T* sd = p.dstd + ((size_t)ti * p.nnei + j) * 4;
    T e4[4] = {(T)0, (T)0, (T)0, (T)0};
    int act = 0;
    double d[3] = {0.0, 0.0, 0.0};
    if (nb >= 0) {
      const int tj = pair_disp(p, f, i, nb, d);
      act = p.pair_mask ? p.pair_mask[ti * p.ntypes + tj] : 1;
      if (act) {
        const T dt[3] = {(T)d[0], (T)d[1], (T)d[2]};
        T der[12];
        env_row<T, false>(dt, rmin, rmax, e4, der);
      }
    } else {
      act = p.pad_zero ? 0 : 1;
    }
#pragma unroll
    for (int c = 0; c < 4; ++c) s_rn[4 * j + c] = (nb >= 0 && !act) ? (T)0 : (e4[c] - av[c]) / sd[c];
    s_act[j] = act;
    if (BWD) {
      s_d[3 * j] = d[0];
      s_d[3 * j + 1] = d[1];
      s_d[3 * j + 2] = d[2];
    }
  }
  __syncthreads();
}

// compact the active slots (in slot order) and record, per type section,
// where its active slots start in the list
__device__ void compact_active(int nnei, int ntypes, const int* sec, const int* s_act, int* s_list,
                               int* s_secpos) {
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    int cnt = 0;
    int t = 0;
    for (int q = 0; q < nnei; q += 32) {
      const int j = q + lane;
      const bool a = j < nnei && s_act[j];
      const unsigned m = __ballot_sync(0xffffffffu, a);
      while (t <= ntypes && sec[t] < q + 32) {
        const int off = sec[t] - q;  // may be <= 0 for sections starting earlier
        const int before = off <= 0 ? 0 : __popc(m & ((off >= 32) ? 0xffffffffu : ((1u << off) - 1u)));
        if (lane == 0) s_secpos[t] = cnt + before;
        ++t;
      }
      if (a) s_list[cnt + __popc(m & ((1u << lane) - 1u))] = j;
      cnt += __popc(m);
    }
    while (t <= ntypes) {
      if (lane == 0) s_secpos[t] = cnt;
      ++t;
    }
  }
  __syncthreads();
}

// one dense layer over a chunk: out[s][o] = tanh(in[s] . W[:, o] + b[o]) * idt
// (+ skip), also storing tanh values when tout != NULL
template <typename T>
__device__ __forceinline__ void dense_layer(int nch, int nin, int nout, const T* __restrict__ W,
                                            const T* __restrict__ b, const T* __restrict__ idt,
                                            const T* in, int ldin, T* out, int ldout, T* tout) {
  for (int q = threadIdx.x; q < nch * nout; q += blockDim.x) {
    const int s = q / nout, o = q - s * nout;
    T acc = __ldg(b + o);
    const T* x = in + s * ldin;
    for (int k = 0; k < nin; ++k) acc += x[k] * __ldg(W + (size_t)k * nout + o);
    const T t = tanh_t<T>(acc);
    T y = idt ? t * __ldg(idt + o) : t;
    if (nout == nin)
      y += x[o];
    else if (nout == 2 * nin)
      y += x[o < nin ? o : o - nin];
    out[s * ldout + o] = y;
    if (tout) tout[s * ldout + o] = t;
  }
}

// ---------------------------------------------------------------------------
template <typename T, int CH>
__global__ void __launch_bounds__(kThreads)
desc_fwd_kernel(DescParams<T> p, EmbParams<T> e, T* __restrict__ Dout, T* __restrict__ xyz_out) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int row = blockIdx.x;
  const int f = row / p.nloc, i = row - f * p.nloc;
  const int ti = p.atype[i];
  const int ng = p.ng;
  const int dim = ng * p.axis;
  const int rpos = p.row_pos[row];
  if (ti < 0) {
    for (int q = threadIdx.x; q < 4 * ng; q += blockDim.x) xyz_out[(size_t)row * 4 * ng + q] = (T)0;
    return;
  }
  const SmemLayout<T> L = make_layout<T, CH, false>(p.nnei, ng, e.n_layer, e.width);
  T* s_rn = reinterpret_cast<T*>(smem + L.rn);
  int* s_act = reinterpret_cast<int*>(smem + L.act);
  int* s_list = reinterpret_cast<int*>(smem + L.list);
  int* s_secpos = reinterpret_cast<int*>(smem + L.secpos);
  T* s_xyz = reinterpret_cast<T*>(smem + L.xyz);
  T* s_xin = reinterpret_cast<T*>(smem + L.xin);
  T* s_buf = reinterpret_cast<T*>(smem + L.buf);
  row_env<T, false>(p, row, f, i, ti, s_rn, s_act, nullptr);
  compact_active(p.nnei, p.ntypes, p.sec, s_act, s_list, s_secpos);

  T acc[kNQ];
#pragma unroll
  for (int k = 0; k < kNQ; ++k) acc[k] = (T)0;
  for (int t = 0; t < p.ntypes; ++t) {
    const int net = p.type_one_side ? t : t * p.ntypes + ti;
    const int a0 = s_secpos[t], a1 = s_secpos[t + 1];
    for (int c0 = a0; c0 < a1; c0 += CH) {
      const int nch = min(CH, a1 - c0);
      const T* G;
      if (e.compressed) {
        const TabMeta<T> tm = e.meta[net];
        T* g = s_buf;
        for (int q = threadIdx.x; q < nch * ng; q += blockDim.x) {
          const int s = q / ng, n = q - s * ng;
          const T x = s_rn[4 * s_list[c0 + s]];
          int idx;
          T xx, delta, val, grad;
          table_locate(tm, x, idx, xx, delta);
          table_poly(e.table + tm.offset + ((size_t)idx * ng + n) * 6, xx, delta, val, grad);
          g[s * kMaxW + n] = val;
        }
        G = g;
      } else {
        for (int s = threadIdx.x; s < nch; s += blockDim.x) s_xin[s] = s_rn[4 * s_list[c0 + s]];
        __syncthreads();
        const T* in = s_xin;
        int ldin = 1, nin = 1;
        for (int l = 0; l < e.n_layer; ++l) {
          const int nout = e.width[l];
          T* out = s_buf + (l & 1) * CH * kMaxW;
          dense_layer<T>(nch, nin, nout, e.W[l] + (size_t)net * nin * nout, e.b[l] + (size_t)net * nout,
                         e.idt[l] ? e.idt[l] + (size_t)net * nout : nullptr, in, ldin, out, kMaxW, nullptr);
          __syncthreads();
          in = out;
          ldin = kMaxW;
          nin = nout;
        }
        G = in;
      }
      __syncthreads();
#pragma unroll
      for (int k = 0; k < kNQ; ++k) {
        const int q = threadIdx.x + k * kThreads;
        if (q < 4 * ng) {
          const int c = q / ng, n = q - c * ng;
          T a = acc[k];
          for (int s = 0; s < nch; ++s) a += s_rn[4 * s_list[c0 + s] + c] * G[s * kMaxW + n];
          acc[k] = a;
        }
      }
      __syncthreads();
    }
  }
  const T inv = (T)1 / (T)p.nnei;
#pragma unroll
  for (int k = 0; k < kNQ; ++k) {
    const int q = threadIdx.x + k * kThreads;
    if (q < 4 * ng) {
      const T v = acc[k] * inv;
      s_xyz[q] = v;
      xyz_out[(size_t)row * 4 * ng + q] = v;
    }
  }
  __syncthreads();
  T* D = Dout + (size_t)rpos * dim;
  for (int q = threadIdx.x; q < dim; q += blockDim.x) {
    const int n = q / p.axis, m = q - n * p.axis;
    T s = (T)0;
#pragma unroll
    for (int c = 0; c < 4; ++c) s += s_xyz[c * ng + n] * s_xyz[c * ng + m];
    D[q] = s;
  }
}

// ---------------------------------------------------------------------------
template <typename T, int CH>
__global__ void __launch_bounds__(kThreads)
desc_bwd_kernel(DescParams<T> p, EmbParams<T> e, const T* __restrict__ dDin,
                const T* __restrict__ xyz_in, T* __restrict__ gpair, double* __restrict__ vir_row) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ double s_vred[kThreads / 32][9];
  const int row = blockIdx.x;
  const int f = row / p.nloc, i = row - f * p.nloc;
  const int ti = p.atype[i];
  const int ng = p.ng, M = p.axis;
  if (ti < 0) {
    for (int q = threadIdx.x; q < 3 * p.nnei; q += blockDim.x) gpair[(size_t)row * 3 * p.nnei + q] = (T)0;
    if (threadIdx.x < 9) vir_row[(size_t)row * 9 + threadIdx.x] = 0.0;
    return;
  }
  const SmemLayout<T> L = make_layout<T, CH, true>(p.nnei, ng, e.n_layer, e.width);
  T* s_rn = reinterpret_cast<T*>(smem + L.rn);
  int* s_act = reinterpret_cast<int*>(smem + L.act);
  int* s_list = reinterpret_cast<int*>(smem + L.list);
  int* s_secpos = reinterpret_cast<int*>(smem + L.secpos);
  double* s_d = reinterpret_cast<double*>(smem + L.dvec);
  T* s_drn = reinterpret_cast<T*>(smem + L.drn);
  T* s_xyz = reinterpret_cast<T*>(smem + L.xyz);
  T* s_dxyz = reinterpret_cast<T*>(smem + L.dxyz);
  T* s_xin = reinterpret_cast<T*>(smem + L.xin);
  T* s_buf = reinterpret_cast<T*>(smem + L.buf);
  // per-layer Y_l, T_l buffers then the three gradient buffers
  T* Ybuf[kMaxEmbLayers];
  T* Tbuf[kMaxEmbLayers];
  {
    T* q = s_buf;
    for (int l = 0; l < e.n_layer; ++l) {
      Ybuf[l] = q;
      q += CH * e.width[l];
      Tbuf[l] = q;
      q += CH * e.width[l];
    }
    s_buf = q;  // the three gradient buffers follow
  }
  T* gA = s_buf;
  T* gB = gA + CH * kMaxW;
  T* gC = gB + CH * kMaxW;

  for (int q = threadIdx.x; q < 4 * ng; q += blockDim.x) s_xyz[q] = xyz_in[(size_t)row * 4 * ng + q];
  row_env<T, true>(p, row, f, i, ti, s_rn, s_act, s_d);  // syncs
  compact_active(p.nnei, p.ntypes, p.sec, s_act, s_list, s_secpos);
  // dE/dxyz (before the 1/nnei of the forward)
  const T* dD = dDin + (size_t)p.row_pos[row] * ng * M;
  const T inv = (T)1 / (T)p.nnei;
  for (int q = threadIdx.x; q < 4 * ng; q += blockDim.x) {
    const int c = q / ng, n = q - c * ng;
    T s = (T)0;
    for (int m = 0; m < M; ++m) s += __ldg(dD + n * M + m) * s_xyz[c * ng + m];
    if (n < M)
      for (int n2 = 0; n2 < ng; ++n2) s += __ldg(dD + n2 * M + n) * s_xyz[c * ng + n2];
    s_dxyz[q] = s * inv;
  }
  for (int q = threadIdx.x; q < 4 * p.nnei; q += blockDim.x) s_drn[q] = (T)0;
  __syncthreads();

  for (int t = 0; t < p.ntypes; ++t) {
    const int net = p.type_one_side ? t : t * p.ntypes + ti;
    const int a0 = s_secpos[t], a1 = s_secpos[t + 1];
    TabMeta<T> tm;
    if (e.compressed) tm = e.meta[net];
    for (int c0 = a0; c0 < a1; c0 += CH) {
      const int nch = min(CH, a1 - c0);
      if (e.compressed) {
        // G and dG/dx from the table; dRn_direct and dss in one pass
        for (int q = threadIdx.x; q < nch * 4; q += blockDim.x) {
          const int s = q >> 2, c = q & 3;
          const int slot = s_list[c0 + s];
          const T x = s_rn[4 * slot];
          int idx;
          T xx, delta;
          table_locate(tm, x, idx, xx, delta);
          T direct = (T)0, dss = (T)0;
          const T r0 = s_rn[4 * slot], r1 = s_rn[4 * slot + 1], r2 = s_rn[4 * slot + 2],
                  r3 = s_rn[4 * slot + 3];
          for (int n = 0; n < ng; ++n) {
            T val, grad;
            table_poly(e.table + tm.offset + ((size_t)idx * ng + n) * 6, xx, delta, val, grad);
            direct += val * s_dxyz[c * ng + n];
            if (c == 0) {
              const T dg = r0 * s_dxyz[n] + r1 * s_dxyz[ng + n] + r2 * s_dxyz[2 * ng + n] +
                           r3 * s_dxyz[3 * ng + n];
              dss += grad * dg;
            }
          }
          s_drn[4 * slot + c] = direct + dss;
        }
        __syncthreads();
        continue;
      }
      // recompute the forward of the chunk, keeping Y_l and tanh T_l
      for (int s = threadIdx.x; s < nch; s += blockDim.x) s_xin[s] = s_rn[4 * s_list[c0 + s]];
      __syncthreads();
      {
        const T* in = s_xin;
        int nin = 1;
        for (int l = 0; l < e.n_layer; ++l) {
          const int nout = e.width[l];
          dense_layer<T>(nch, nin, nout, e.W[l] + (size_t)net * nin * nout, e.b[l] + (size_t)net * nout,
                         e.idt[l] ? e.idt[l] + (size_t)net * nout : nullptr, in, nin, Ybuf[l], nout, Tbuf[l]);
          __syncthreads();
          in = Ybuf[l];
          nin = nout;
        }
      }
      const T* G = Ybuf[e.n_layer - 1];
      // dRn_direct[s][c] = sum_n G[s][n] dxyz[c][n];  dG[s][n] = sum_c Rn[s][c] dxyz[c][n]
      for (int q = threadIdx.x; q < nch * 4; q += blockDim.x) {
        const int s = q >> 2, c = q & 3;
        T a = (T)0;
        for (int n = 0; n < ng; ++n) a += G[s * ng + n] * s_dxyz[c * ng + n];
        s_drn[4 * s_list[c0 + s] + c] = a;
      }
      for (int q = threadIdx.x; q < nch * ng; q += blockDim.x) {
        const int s = q / ng, n = q - s * ng;
        const int slot = s_list[c0 + s];
        gA[s * kMaxW + n] = s_rn[4 * slot] * s_dxyz[n] + s_rn[4 * slot + 1] * s_dxyz[ng + n] +
                            s_rn[4 * slot + 2] * s_dxyz[2 * ng + n] + s_rn[4 * slot + 3] * s_dxyz[3 * ng + n];
      }
      __syncthreads();
      // back-propagate through the layers; gA holds dY of layer l
      T* dY = gA;
      T* dP = gB;
      T* dX = gC;
      for (int l = e.n_layer - 1; l >= 0; --l) {
        const int nout = e.width[l];
        const int nin = l == 0 ? 1 : e.width[l - 1];
        const T* idt = e.idt[l] ? e.idt[l] + (size_t)net * nout : nullptr;
        const T* W = e.W[l] + (size_t)net * nin * nout;
        for (int q = threadIdx.x; q < nch * nout; q += blockDim.x) {
          const int s = q / nout, o = q - s * nout;
          const T tv = Tbuf[l][s * nout + o];
          dP[s * kMaxW + o] = dY[s * kMaxW + o] * (idt ? __ldg(idt + o) : (T)1) * ((T)1 - tv * tv);
        }
        __syncthreads();
        for (int q = threadIdx.x; q < nch * nin; q += blockDim.x) {
          const int s = q / nin, k = q - s * nin;
          T a = (T)0;
          for (int o = 0; o < nout; ++o) a += dP[s * kMaxW + o] * __ldg(W + (size_t)k * nout + o);
          if (nout == nin)
            a += dY[s * kMaxW + k];
          else if (nout == 2 * nin)
            a += dY[s * kMaxW + k] + dY[s * kMaxW + k + nin];
          dX[s * kMaxW + k] = a;
        }
        __syncthreads();
        T* tmp = dY;
        dY = dX;
        dX = tmp;
      }
      for (int s = threadIdx.x; s < nch; s += blockDim.x) s_drn[4 * s_list[c0 + s]] += dY[s * kMaxW];
      __syncthreads();
    }
  }
  // pair gradient g = dE/d(r_j - r_i) and the centre-side virial
  double v[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) v[k] = 0.0;
  const T rmin = (T)p.rcut_smth, rmax = (T)p.rcut;
  for (int j = threadIdx.x; j < p.nnei; j += blockDim.x) {
    const int nb = p.nlist[(size_t)row * p.nnei + j];
    T g[3] = {(T)0, (T)0, (T)0};
    if (nb >= 0 && s_act[j]) {
      const double* d = s_d + 3 * j;
      const T dt[3] = {(T)d[0], (T)d[1], (T)d[2]};
      T em[4], der[12];
      env_row<T, true>(dt, rmin, rmax, em, der);
      const T* sd = p.dstd + ((size_t)ti * p.nnei + j) * 4;
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const T w = s_drn[4 * j + c] / sd[c];
#pragma unroll
        for (int k = 0; k < 3; ++k) g[k] -= w * der[3 * c + k];
      }
#pragma unroll
      for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int l2 = 0; l2 < 3; ++l2) v[3 * k + l2] -= (double)g[k] * d[l2];
    }
    T* gp = gpair + ((size_t)row * p.nnei + j) * 3;
    gp[0] = g[0];
    gp[1] = g[1];
    gp[2] = g[2];
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    const double w = warp_sum(v[k]);
    if (lane == 0) s_vred[warp][k] = w;
  }
  __syncthreads();
  if (threadIdx.x < 9) {
    double s = 0.0;
    for (int w = 0; w < kThreads / 32; ++w) s += s_vred[w][threadIdx.x];
    vir_row[(size_t)row * 9 + threadIdx.x] = s;
  }
}

template <typename T>
constexpr int chunk_of() {
  return sizeof(T) == 8 ? 16 : 32;
}

}  // namespace

template <typename T>
size_t desc_fwd_smem(const DescParams<T>& p, const EmbParams<T>& e) {
  return make_layout<T, chunk_of<T>(), false>(p.nnei, p.ng, e.n_layer, e.width).total;
}
template <typename T>
size_t desc_bwd_smem(const DescParams<T>& p, const EmbParams<T>& e) {
  return make_layout<T, chunk_of<T>(), true>(p.nnei, p.ng, e.n_layer, e.width).total;
}

template <typename T>
int launch_desc_fwd(const DescParams<T>& p, const EmbParams<T>& e, T* D, T* xyz, size_t smem,
                    cudaStream_t st) {
  if (p.nrows <= 0) return DPGB_OK;
  auto kern = desc_fwd_kernel<T, chunk_of<T>()>;
  DPGB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  kern<<<p.nrows, kThreads, smem, st>>>(p, e, D, xyz);
  return check_launch("desc_fwd");
}

template <typename T>
int launch_desc_bwd(const DescParams<T>& p, const EmbParams<T>& e, const T* dD, const T* xyz, T* gpair,
                    double* vir_row, size_t smem, cudaStream_t st) {
  if (p.nrows <= 0) return DPGB_OK;
  auto kern = desc_bwd_kernel<T, chunk_of<T>()>;
  DPGB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  kern<<<p.nrows, kThreads, smem, st>>>(p, e, dD, xyz, gpair, vir_row);
  return check_launch("desc_bwd");
}

template size_t desc_fwd_smem<double>(const DescParams<double>&, const EmbParams<double>&);
template size_t desc_fwd_smem<float>(const DescParams<float>&, const EmbParams<float>&);
template size_t desc_bwd_smem<double>(const DescParams<double>&, const EmbParams<double>&);
template size_t desc_bwd_smem<float>(const DescParams<float>&, const EmbParams<float>&);
template int launch_desc_fwd<double>(const DescParams<double>&, const EmbParams<double>&, double*, double*,
                                     size_t, cudaStream_t);
template int launch_desc_fwd<float>(const DescParams<float>&, const EmbParams<float>&, float*, float*, size_t,
                                    cudaStream_t);
template int launch_desc_bwd<double>(const DescParams<double>&, const EmbParams<double>&, const double*,
                                     const double*, double*, double*, size_t, cudaStream_t);
template int launch_desc_bwd<float>(const DescParams<float>&, const EmbParams<float>&, const float*,
                                    const float*, float*, double*, size_t, cudaStream_t);

}  // namespace dpgb
