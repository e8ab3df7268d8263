// Tensor-core se_e2_a embedding (mixed precision): the two dense layers of
// the 1 -> w1 -> w2 -> w3 embedding net (and their input-gradient products in
// the backward pass) run as tcgen05.mma with BF16 operands in shared memory
// and FP32 accumulators in TMEM; the tanh epilogues, the per-atom contraction
// xyz = sum_j R~_j^T G_j and the force products run on the CUDA cores in
// FP32.  G itself is never rounded to BF16: it is formed in FP32 from the
// FP32 accumulator and contracted in FP32.
//
// Work decomposition: a persistent CTA owns contiguous ranges of type-sorted
// atoms of one centre type.  For each neighbour-type section it packs whole
// per-atom runs of active slots into tiles of up to 128 pairs (= the 128 TMEM
// lanes / MMA rows) and at most 16 atoms, so every atom's xyz and virial are
// accumulated by one CTA in a fixed order: no atomics, bitwise reproducible.
// Semantics follow deepmd/pt/model/descriptor/se_a.py:742-858 and
// env_mat.py:18-119 (padding slots hold (0 - avg)/std and go through the net
// unless avg == 0; excluded pairs contribute zero).
#include <cstring>
#include <vector>

#include "emb_tc.cuh"
#include "tc.cuh"

namespace dpgb {

static inline int pad16(int x) { return (x + 15) / 16 * 16; }

int emb_tc_eligible(const dpgb_se_a_desc& d) {
  if (d.compressed || d.n_emb != 3) return 0;
  const int w1 = d.emb_neuron[0], w2 = d.emb_neuron[1], w3 = d.emb_neuron[2];
  const bool shape_a = (w1 == 25 && w2 == 50 && w3 == 100);
  const bool shape_b = (w1 == 3 && w2 == 6 && w3 == 12);
  if (!shape_a && !shape_b) return 0;
  // two spare padding columns after layers 1 and 2 carry the biases
  if (pad16(w1) - w1 < 2 || bias_col(1, w2, w1, pad16(w2)) < 0) return 0;
  for (int t = 0; t < d.ntypes; ++t)
    if (d.sel[t] > kTcRows) return 0;
  return 1;
}

size_t emb_tc_image_bytes(const EmbTC& m, int kind) {
  switch (kind) {
    case 0: case 4: return (size_t)m.n2 * m.k1 * 2;
    case 1: case 5: return (size_t)m.n3 * m.n2 * 2;
    case 2: return (size_t)m.n2 * m.n3 * 2;
    default: return (size_t)m.k1 * m.n2 * 2;
  }
}
constexpr int kEmbImageKinds = 6;

static void put_bf16(std::vector<unsigned char>& img, size_t base, int r, int k, int K, float v) {
  const __nv_bfloat16 b = __float2bfloat16_rn(v);
  std::memcpy(img.data() + base + tc::cm_offset(r, k, K), &b, 2);
}

// the low BF16 part of a weight (its remainder after the BF16 rounding)
static float bf16_lo(double w) {
  const __nv_bfloat16 hi = __float2bfloat16_rn((float)w);
  return (float)(w - (double)__bfloat162float(hi));
}

// bias b of output row r as BF16 hi + lo on the K columns k_hi, k_lo (the
// operand holds 1 there)
static void put_bias(std::vector<unsigned char>& img, size_t base, int r, int k_hi, int k_lo, int K, double b) {
  const __nv_bfloat16 hi = __float2bfloat16_rn((float)b);
  put_bf16(img, base, r, k_hi, K, (float)b);
  put_bf16(img, base, r, k_lo, K, (float)(b - (double)__bfloat162float(hi)));
}

int build_emb_tc(const dpgb_se_a_desc& d, std::vector<unsigned char>& images, EmbTC& m, std::vector<float>& vec) {
  const int nnets = d.type_one_side ? d.ntypes : d.ntypes * d.ntypes;
  m.w1 = d.emb_neuron[0];
  m.w2 = d.emb_neuron[1];
  m.w3 = d.emb_neuron[2];
  m.k1 = pad16(m.w1);
  m.n2 = pad16(m.w2);
  m.n3 = pad16(m.w3);
  m.nnets = nnets;
  m.vec_stride = 3 * m.k1 + 2 * m.n2 + 2 * m.n3;
  size_t per[kEmbImageKinds], kind0[kEmbImageKinds + 1] = {0};
  for (int k = 0; k < kEmbImageKinds; ++k) {
    per[k] = emb_tc_image_bytes(m, k);
    kind0[k + 1] = kind0[k] + per[k] * nnets;  // images of kind k: nets in order from kind0[k]
  }
  images.assign(kind0[kEmbImageKinds], 0);
  vec.assign((size_t)m.vec_stride * nnets, 0.f);
  m.has_idt1 = m.has_idt2 = m.has_idt3 = 0;
  for (int e = 0; e < nnets; ++e) {
    const double* W1 = d.emb_w[e][0];  // [1, w1]
    const double* W2 = d.emb_w[e][1];  // [w1, w2]
    const double* W3 = d.emb_w[e][2];  // [w2, w3]
    if (!W1 || !W2 || !W3 || !d.emb_b[e][0] || !d.emb_b[e][1] || !d.emb_b[e][2]) return fail(DPGB_EINVAL, "missing embedding weights");
    const size_t b0 = kind0[0] + per[0] * e, b1 = kind0[1] + per[1] * e, b2 = kind0[2] + per[2] * e,
                 b3 = kind0[3] + per[3] * e, b4 = kind0[4] + per[4] * e, b5 = kind0[5] + per[5] * e;
    // layer-2 outputs o sit at column c2 = neuron_col(o), layer-3 outputs at
    // c3; the biases of layers 2 and 3 on the bias columns of their inputs
    const int k2a = m.w1, k2b = m.w1 + 1;
    const int k3a = bias_col(0, m.w2, m.w1, m.n2), k3b = bias_col(1, m.w2, m.w1, m.n2);
    for (int o = 0; o < m.w2; ++o)
      put_bias(images, b0, neuron_col(o, m.w2, m.w1), k2a, k2b, m.k1, d.emb_b[e][1][o]);
    for (int o = 0; o < m.w3; ++o)
      put_bias(images, b1, neuron_col(o, m.w3, m.w2), k3a, k3b, m.n2, d.emb_b[e][2][o]);
    for (int o = 0; o < m.w2; ++o)
      for (int k = 0; k < m.w1; ++k) {
        const int c2 = neuron_col(o, m.w2, m.w1);
        put_bf16(images, b0, c2, k, m.k1, (float)W2[(size_t)k * m.w2 + o]);  // W2^T [n2 x k1]
        put_bf16(images, b4, c2, k, m.k1, bf16_lo(W2[(size_t)k * m.w2 + o]));
        put_bf16(images, b3, k, c2, m.n2, (float)W2[(size_t)k * m.w2 + o]);  // W2 [k1 x n2]
      }
    for (int o = 0; o < m.w3; ++o)
      for (int k = 0; k < m.w2; ++k) {
        const int c3 = neuron_col(o, m.w3, m.w2), c2 = neuron_col(k, m.w2, m.w1);
        put_bf16(images, b1, c3, c2, m.n2, (float)W3[(size_t)k * m.w3 + o]);  // W3^T [n3 x n2]
        put_bf16(images, b5, c3, c2, m.n2, bf16_lo(W3[(size_t)k * m.w3 + o]));
        put_bf16(images, b2, c2, c3, m.n3, (float)W3[(size_t)k * m.w3 + o]);  // W3 [n2 x n3]
      }
    float* v = vec.data() + (size_t)m.vec_stride * e;
    for (int k = 0; k < m.w1; ++k) {
      v[k] = (float)W1[k];
      v[m.k1 + k] = (float)d.emb_b[e][0][k];
      v[2 * m.k1 + k] = d.emb_idt[e][0] ? (float)d.emb_idt[e][0][k] : 1.f;
    }
    float* v2 = v + 3 * m.k1;
    for (int o = 0; o < m.w2; ++o) {
      const int c2 = neuron_col(o, m.w2, m.w1);
      v2[c2] = (float)d.emb_b[e][1][o];
      v2[m.n2 + c2] = d.emb_idt[e][1] ? (float)d.emb_idt[e][1][o] : 1.f;
    }
    float* v3 = v2 + 2 * m.n2;
    for (int o = 0; o < m.w3; ++o) {
      const int c3 = neuron_col(o, m.w3, m.w2);
      v3[c3] = (float)d.emb_b[e][2][o];
      v3[m.n3 + c3] = d.emb_idt[e][2] ? (float)d.emb_idt[e][2][o] : 1.f;
    }
    m.has_idt1 |= d.emb_idt[e][0] != nullptr;
    m.has_idt2 |= d.emb_idt[e][1] != nullptr;
    m.has_idt3 |= d.emb_idt[e][2] != nullptr;
  }
  return DPGB_OK;
}

void emb_tc_bind(EmbTC& m, const unsigned char* dev, size_t, const float* dev_vec) {
  const unsigned char** dst[kEmbImageKinds] = {&m.fw2, &m.fw3, &m.bw3, &m.bw2, &m.fw2lo, &m.fw3lo};
  size_t off = 0;
  for (int k = 0; k < kEmbImageKinds; ++k) {
    *dst[k] = dev + off;
    off += emb_tc_image_bytes(m, k) * m.nnets;
  }
  m.vec = dev_vec;
}

namespace {

__device__ __forceinline__ float tanh_fast(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// copy a net's weight image (bytes multiple of 16) into shared memory
__device__ __forceinline__ void copy16(unsigned char* dst, const unsigned char* src, int bytes) {
  for (int q = threadIdx.x; q < bytes / 16; q += blockDim.x)
    reinterpret_cast<uint4*>(dst)[q] = reinterpret_cast<const uint4*>(src)[q];
}

// store 8 consecutive bf16 values of row r, columns k0..k0+7, in the
// core-matrix layout of a tile with K columns
__device__ __forceinline__ void store8(unsigned char* base, int r, int k0, int K, const float* v) {
  __nv_bfloat162 h[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) h[i] = __floats2bfloat162_rn(v[2 * i], v[2 * i + 1]);
  *reinterpret_cast<uint4*>(base + tc::cm_offset(r, k0, K)) = *reinterpret_cast<uint4*>(h);
}

// the same as split-BF16 parts: the high parts (BF16 of v) at base, the low
// parts (BF16 of v - hi) at base_lo; an MMA over each then carries the
// operand to ~16 significant bits (1 and 0 have no low part)
__device__ __forceinline__ void store8_split(unsigned char* base, unsigned char* base_lo, int r, int k0, int K,
                                             const float* v) {
  __nv_bfloat162 h[4], l[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    h[i] = __floats2bfloat162_rn(v[2 * i], v[2 * i + 1]);
    l[i] = __floats2bfloat162_rn(v[2 * i] - __low2float(h[i]), v[2 * i + 1] - __high2float(h[i]));
  }
  const int off = tc::cm_offset(r, k0, K);
  *reinterpret_cast<uint4*>(base + off) = *reinterpret_cast<uint4*>(h);
  *reinterpret_cast<uint4*>(base_lo + off) = *reinterpret_cast<uint4*>(l);
}

// D (+)= A B over kdim; acc0: add onto what D holds already (a preloaded
// residual term) instead of overwriting it in the first step
template <int K1, int N>
__device__ __forceinline__ void issue_mma(uint32_t d_tmem, uint32_t a_s, uint32_t b_s, int kdim, bool acc0 = false) {
  const uint32_t idesc = tc::idesc_bf16_f32(128, N);
  const uint32_t sbo = (uint32_t)(kdim / 8) * 128;
  for (int ks = 0; ks < kdim / 16; ++ks)
    tc::mma_bf16(d_tmem, tc::smem_desc(a_s + ks * 256, 128, sbo), tc::smem_desc(b_s + ks * 256, 128, sbo), idesc,
                 (ks > 0 || acc0) ? 1u : 0u);
}

// Pack whole runs of section t (rows s_cursor .. row1 of the type-sorted
// order) into one tile of at most kTcRows pairs and kMaxAtoms atoms.  Warp 0
// loads 32 run lengths (and rows) at once and every lane runs the same greedy
// loop over them through shuffles, so one load round trip serves up to 32
// rows instead of one dependent load per row.
template <int kMaxAtoms>
__device__ __forceinline__ void pack_tile(const int* __restrict__ run_len, const int* __restrict__ sorted_rows,
                                          int ntypes, int row1, int t, int* s_row, int* s_off, int* s_ntile,
                                          int* s_cursor, int lane) {
  int cur = *s_cursor, n = 0, pairs = 0;
  bool done = false;
  while (!done && cur < row1) {
    const int r = cur + lane;
    const int len = r < row1 ? run_len[(size_t)r * ntypes + t] : -1;
    const int srow = r < row1 ? sorted_rows[r] : 0;
    int k = 0;
    for (; k < 32; ++k) {
      const int lk = __shfl_sync(0xffffffffu, len, k);
      const int sk = __shfl_sync(0xffffffffu, srow, k);
      if (lk < 0 || (lk > 0 && (n == kMaxAtoms || pairs + lk > kTcRows))) {
        done = true;
        break;
      }
      if (lk == 0) continue;
      if (lane == 0) {
        s_row[n] = sk;
        s_off[n] = pairs;
      }
      pairs += lk;
      ++n;
    }
    cur += k;
  }
  if (lane == 0) {
    s_off[n] = pairs;
    *s_ntile = n;
    *s_cursor = cur;
  }
}

// TMEM columns [c0, c0 + 32) of this warp's 32 lanes (the second 16 only
// when they exist in an NCOL-column accumulator) with one wait for both
template <int NCOL>
__device__ __forceinline__ void tmem_ld32(uint32_t lane_base, int c0, float (&v)[32]) {
  tc::tmem_ld16(lane_base + c0, *reinterpret_cast<float(*)[16]>(v));
  if (c0 + 16 < NCOL) tc::tmem_ld16(lane_base + c0 + 16, *reinterpret_cast<float(*)[16]>(v + 16));
  tc::tmem_ld_wait();
}

// Environment of the tile's pair p: fills Rn (normalised), d (displacement,
// FP32 after the FP64 subtraction), the slot index and flags.
struct PairInfo {
  int row, slot, nb, keep, valid, k;
};

__device__ __forceinline__ void pair_env(const DescParams<float>& p, int t, int ti, const int* s_row,
                                         const int* s_off, int ntile, int pp, PairInfo& pi, float rn[4],
                                         float dvec[3]) {
  pi.valid = pp < s_off[ntile];
  rn[0] = rn[1] = rn[2] = rn[3] = 0.f;
  dvec[0] = dvec[1] = dvec[2] = 0.f;
  pi.nb = -1;
  pi.keep = 0;
  pi.k = 0;
  pi.row = 0;
  pi.slot = 0;
  if (!pi.valid) return;
  int k = 0;
  while (k + 1 < ntile && s_off[k + 1] <= pp) ++k;
  pi.k = k;
  pi.row = s_row[k];
  pi.slot = p.sec[t] + (pp - s_off[k]);
  const int f = p.nloc_div.div(pi.row), i = pi.row - f * p.nloc;
  pi.nb = p.nlist[(size_t)pi.row * p.nnei + pi.slot];
  const float* av = p.davg + ((size_t)ti * p.nnei + pi.slot) * 4;
  const float* sdi = p.dstd_inv + ((size_t)ti * p.nnei + pi.slot) * 4;
  float e4[4] = {0.f, 0.f, 0.f, 0.f};
  if (pi.nb >= 0) {
    const int tj = pair_disp_f(p, f, i, pi.nb, dvec);
    pi.keep = p.pair_mask ? p.pair_mask[ti * p.ntypes + tj] : 1;
    if (pi.keep) {
      const float nr2 = dvec[0] * dvec[0] + dvec[1] * dvec[1] + dvec[2] * dvec[2];
      const float nr = sqrtf(nr2);
      const float inr = 1.f / nr;
      const float rmin = (float)p.rcut_smth, rmax = (float)p.rcut;
      float sw;
      if (nr < rmin) {
        sw = 1.f;
      } else if (nr < rmax) {
        const float uu = (nr - rmin) / (rmax - rmin);
        sw = uu * uu * uu * (-6.f * uu * uu + 15.f * uu - 10.f) + 1.f;
      } else {
        sw = 0.f;
      }
      const float inr2 = inr * inr;
      e4[0] = inr * sw;
      e4[1] = dvec[0] * inr2 * sw;
      e4[2] = dvec[1] * inr2 * sw;
      e4[3] = dvec[2] * inr2 * sw;
    }
  }
#pragma unroll
  for (int c = 0; c < 4; ++c) rn[c] = (pi.nb >= 0 && !pi.keep) ? 0.f : (e4[c] - av[c]) * sdi[c];
}

// d R~ / d r_centre of a kept pair (env_mat.cc:156-216), FP32
__device__ __forceinline__ void env_deriv(const float d[3], float rmin, float rmax, float der[12]) {
  const float nr2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
  const float nr = sqrtf(nr2);
  const float inr = 1.f / nr;
  float sw, dsw;
  if (nr < rmin) {
    sw = 1.f;
    dsw = 0.f;
  } else if (nr < rmax) {
    const float du = 1.f / (rmax - rmin);
    const float uu = (nr - rmin) * du;
    const float poly = -6.f * uu * uu + 15.f * uu - 10.f;
    sw = uu * uu * uu * poly + 1.f;
    dsw = (3.f * uu * uu * poly + uu * uu * uu * (-12.f * uu + 15.f)) * du;
  } else {
    sw = 0.f;
    dsw = 0.f;
  }
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
// shared-memory plan (bytes), identical for forward and backward where shared
constexpr int kFinAtoms = 4;  // atoms finalised together (xyz -> D) in the forward

// shared-memory plans (bytes).  Operands that are never live at the same
// time share one region: in the forward A1 (read by the layer-2 MMA, done
// before A2 is written), A2 (read by the layer-3 MMA, done before G is
// written), G and the finalize staging.  Together with 128 TMEM columns (the
// layer-3 accumulator reuses the layer-2 columns once they are read) three
// CTAs fit on an SM for the 25/50/100 net.
template <int W1, int W2, int W3>
struct PlanF {
  static constexpr int K1 = (W1 + 15) / 16 * 16, N2 = (W2 + 15) / 16 * 16, N3 = (W3 + 15) / 16 * 16;
  // G is staged in FP32 by accumulator column, HC columns per pass (row
  // stride LDG; a row's float4 quad q sits at quad q ^ (row & 7), so the
  // eight rows of a float4 store phase hit distinct banks)
  static constexpr int HC = 64, LDG = HC;
  // operand columns holding 1 for the biases of layers 2 (A1) and 3 (A2)
  static constexpr int ONE2a = W1, ONE2b = W1 + 1, ONE3a = bias_col(0, W2, W1, N2), ONE3b = bias_col(1, W2, W1, N2);
  static constexpr int VEC = 3 * K1 + 2 * N2 + 2 * N3;
  // weights in split BF16: the high parts, then the low parts
  static constexpr int fw2 = 0;
  static constexpr int fw3 = fw2 + N2 * K1 * 2;
  static constexpr int fw2lo = fw3 + N3 * N2 * 2;
  static constexpr int fw3lo = fw2lo + N2 * K1 * 2;
  static constexpr int vec = fw3lo + N3 * N2 * 2;
  static constexpr int rn = (vec + VEC * 4 + 15) / 16 * 16;
  static constexpr int reg = (rn + 128 * 4 * 4 + 127) / 128 * 128;
  // split-BF16 operands: the low parts follow the high parts
  static constexpr int a1 = reg, a1lo = reg + 128 * K1 * 2, a2 = reg, a2lo = reg + 128 * N2 * 2;
  static constexpr int gbuf = reg, xs = reg;
  static constexpr int cmax(int a, int b) { return a > b ? a : b; }
  static constexpr int reg_bytes =
      cmax(cmax(2 * 128 * K1 * 2, 2 * 128 * N2 * 2), cmax(128 * LDG * 4, kFinAtoms * 4 * W3 * 4));
  static constexpr int total = reg + reg_bytes;
  static constexpr int tmem_cols = cmax(N2, N3) <= 128 ? 128 : 256;
};
// Backward: A1, A2, dP3, dP2 and the per-pair virial take turns in one region
// (each is written after the MMA that read its predecessor completed); the
// atoms' dE/dxyz are read through L1.  TMEM (128 columns): the layer-2 and
// layer-3 accumulators at column 0 (in turn), dH2 at 0 and dH1 at n2, both
// preloaded with their residual terms so that their MMAs add onto them.
template <int W1, int W2, int W3>
struct PlanB {
  static constexpr int K1 = (W1 + 15) / 16 * 16, N2 = (W2 + 15) / 16 * 16, N3 = (W3 + 15) / 16 * 16;
  static constexpr int VEC = 3 * K1 + 2 * N2 + 2 * N3;
  static constexpr int ONE2a = W1, ONE2b = W1 + 1, ONE3a = bias_col(0, W2, W1, N2), ONE3b = bias_col(1, W2, W1, N2);
  static constexpr int fw2 = 0;
  static constexpr int fw3 = fw2 + N2 * K1 * 2;
  static constexpr int bw3 = fw3 + N3 * N2 * 2;
  static constexpr int bw2 = bw3 + N2 * N3 * 2;
  static constexpr int vec = bw2 + K1 * N2 * 2;
  static constexpr int reg = (vec + VEC * 4 + 127) / 128 * 128;
  // the recomputed forward's operands are split-BF16 (low parts after the
  // high parts), as in the forward; the gradient operands dP3, dP2 are BF16
  static constexpr int a1 = reg, a1lo = reg + 128 * K1 * 2, a2 = reg, a2lo = reg + 128 * N2 * 2, a3 = reg, vir = reg;
  static constexpr int cmax(int a, int b) { return a > b ? a : b; }
  static constexpr int reg_bytes = cmax(cmax(2 * 128 * K1 * 2, 2 * 128 * N2 * 2), cmax(128 * N3 * 2, 128 * 12 * 4));
  static constexpr int total = reg + reg_bytes;
  static constexpr int tmem_cols = cmax(N3, N2 + K1) <= 128 ? 128 : 256;
};

template <int W1, int W2, int W3, bool IDT>
__global__ void __launch_bounds__(128, 3)
emb_tc_fwd_kernel(DescParams<float> p, EmbTC e, const WorkChunk* __restrict__ chunks, int nchunks,
                  const int* __restrict__ run_len, const int* __restrict__ sorted_rows, float* __restrict__ xyz,
                  float* __restrict__ xyzp, float* __restrict__ Dout, int* __restrict__ status,
                  int* __restrict__ queue) {
  using P = PlanF<W1, W2, W3>;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ uint64_t bar;
  __shared__ uint32_t s_tmem;
  __shared__ int s_row[kTcMaxAtoms], s_off[kTcMaxAtoms + 1], s_ntile, s_cursor;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int ng = p.ng;
  if (warp == 0) tc::tmem_alloc(&s_tmem, P::tmem_cols);
  if (tid == 0) tc::mbar_init(&bar, 1);
  __syncthreads();
  tc::fence_after();
  const uint32_t tbase = s_tmem;
  uint32_t phase = 0;
  bool alive = true;
  float* sG = reinterpret_cast<float*>(smem + P::gbuf);
  float* sRn = reinterpret_cast<float*>(smem + P::rn);
  float* sV = reinterpret_cast<float*>(smem + P::vec);
  const uint32_t sA1 = tc::smem_u32(smem + P::a1), sA2 = tc::smem_u32(smem + P::a2);
  const uint32_t sA1lo = tc::smem_u32(smem + P::a1lo), sA2lo = tc::smem_u32(smem + P::a2lo);
  const uint32_t sW2 = tc::smem_u32(smem + P::fw2), sW3 = tc::smem_u32(smem + P::fw3);
  const uint32_t sW2lo = tc::smem_u32(smem + P::fw2lo), sW3lo = tc::smem_u32(smem + P::fw3lo);
  __shared__ int s_work;
  for (int c = work_first(queue, &s_work); c < nchunks && alive; c = work_next(queue, c, &s_work)) {
    const WorkChunk ch = chunks[c];
    const int ti = ch.ti;
    for (int t = 0; t < p.ntypes && alive; ++t) {
      const int net = p.type_one_side ? t : t * p.ntypes + ti;
      float* xpart = xyzp + (size_t)t * p.nrows * 4 * P::N3;  // this section's partial xyz, by column
      copy16(smem + P::fw2, e.fw2 + (size_t)net * P::N2 * P::K1 * 2, P::N2 * P::K1 * 2);
      copy16(smem + P::fw3, e.fw3 + (size_t)net * P::N3 * P::N2 * 2, P::N3 * P::N2 * 2);
      copy16(smem + P::fw2lo, e.fw2lo + (size_t)net * P::N2 * P::K1 * 2, P::N2 * P::K1 * 2);
      copy16(smem + P::fw3lo, e.fw3lo + (size_t)net * P::N3 * P::N2 * 2, P::N3 * P::N2 * 2);
      for (int q = tid; q < P::VEC; q += blockDim.x) sV[q] = e.vec[(size_t)net * P::VEC + q];
      if (tid == 0) s_cursor = ch.row0;
      __syncthreads();
      const float* w1 = sV;
      const float* b1 = sV + P::K1;
      const float* i1 = sV + 2 * P::K1;
      const float* b2 = sV + 3 * P::K1;
      const float* i2 = b2 + P::N2;
      const float* b3 = i2 + P::N2;
      const float* i3 = b3 + P::N3;
      while (alive) {
        // pack whole runs of this section into a tile
        if (warp == 0)
          pack_tile<kTcMaxAtoms>(run_len, sorted_rows, p.ntypes, ch.row1, t, s_row, s_off, &s_ntile, &s_cursor, tid & 31);
        __syncthreads();
        const int ntile = s_ntile;
        if (ntile == 0) break;
        // pair environment and layer 1 (1 -> W1) on the CUDA cores
        PairInfo pi;
        float rn[4], dv[3];
        pair_env(p, t, ti, s_row, s_off, ntile, tid, pi, rn, dv);
#pragma unroll
        for (int cc = 0; cc < 4; ++cc) sRn[tid * 4 + cc] = rn[cc];
        const float x = rn[0];
        float h1[W1];
#pragma unroll
        for (int k = 0; k < W1; ++k) {
          // rows past the tile's pairs carry finite values no output reads
          float h = tanh_fast(fmaf(x, w1[k], b1[k]));
          if (IDT) h *= i1[k];
          if (W1 == 1 || W1 == 2) h += x;
          h1[k] = h;
        }
#pragma unroll
        for (int k0 = 0; k0 < P::K1; k0 += 8) {
          float v[8];
#pragma unroll
          for (int i = 0; i < 8; ++i)
            v[i] = (k0 + i < W1) ? h1[k0 + i] : (k0 + i == P::ONE2a || k0 + i == P::ONE2b ? 1.f : 0.f);
          store8_split(smem + P::a1, smem + P::a1lo, tid, k0, P::K1, v);
        }
        tc::fence_async_smem();
        __syncthreads();
        tc::fence_after();
        if (tid == 0) {
          issue_mma<P::K1, P::N2>(tbase, sA1, sW2, P::K1);  // hi.hi + lo.hi + hi.lo
          issue_mma<P::K1, P::N2>(tbase, sA1lo, sW2, P::K1, true);
          issue_mma<P::K1, P::N2>(tbase, sA1, sW2lo, P::K1, true);
          tc::mma_commit(&bar);
        }
        bool ok = tc::mbar_wait(&bar, phase, status + kStatusTimeout);
        phase ^= 1;
        tc::fence_after();
        // epilogue 2: H2 = tanh(acc) * idt2 + skip(H1) (acc includes b2)
        float h2[W2];
#pragma unroll
        for (int c0 = 0; c0 < P::N2; c0 += 32) {
          float v[32];
          tmem_ld32<P::N2>(tc::taddr(tbase, warp * 32, 0), c0, v);
#pragma unroll
          for (int i = 0; i < 32; ++i) {
            const int c = c0 + i, o = c < P::N2 ? col_neuron(c, W2, W1) : -1;
            if (o >= 0) {
              float h = tanh_fast(v[i]);
              if (IDT) h *= i2[c];
              if (W2 == W1) h += h1[o];
              if (W2 == 2 * W1) h += h1[o < W1 ? o : o - W1];
              h2[o] = h;
            }
          }
        }
#pragma unroll
        for (int k0 = 0; k0 < P::N2; k0 += 8) {
          float v[8];
#pragma unroll
          for (int i = 0; i < 8; ++i) {
            const int o = col_neuron(k0 + i, W2, W1);
            v[i] = o >= 0 ? h2[o] : (k0 + i == P::ONE3a || k0 + i == P::ONE3b ? 1.f : 0.f);
          }
          store8_split(smem + P::a2, smem + P::a2lo, tid, k0, P::N2, v);
        }
        tc::fence_before();
        tc::fence_async_smem();
        __syncthreads();
        tc::fence_after();
        if (tid == 0) {
          issue_mma<P::N2, P::N3>(tbase, sA2, sW3, P::N2);  // over the consumed layer-2 columns
          issue_mma<P::N2, P::N3>(tbase, sA2lo, sW3, P::N2, true);
          issue_mma<P::N2, P::N3>(tbase, sA2, sW3lo, P::N2, true);
          tc::mma_commit(&bar);
        }
        ok = tc::mbar_wait(&bar, phase, status + kStatusTimeout) && ok;
        phase ^= 1;
        tc::fence_after();
        // epilogue 3: G = tanh(acc) * idt3 + skip(H2) (acc includes b3), kept in FP32,
        // staged and contracted HC accumulator columns at a time
#pragma unroll
        for (int cb = 0; cb < P::N3; cb += P::HC) {  // unrolled: column indices stay compile-time
          if (!alive) break;
          // G of columns [cb, cb + HC) by column (0 on padding columns)
#pragma unroll
          for (int c0 = 0; c0 < P::HC; c0 += 16) {
            if (cb + c0 >= P::N3) break;
            float v[16], g[16];
            tc::tmem_ld16(tc::taddr(tbase, warp * 32, cb + c0), v);
            tc::tmem_ld_wait();
#pragma unroll
            for (int i = 0; i < 16; ++i) {
              const int c = cb + c0 + i, o = col_neuron(c, W3, W2);
              g[i] = 0.f;
              if (o >= 0) {
                float x3 = tanh_fast(v[i]);
                if (IDT) x3 *= i3[c];
                if (W3 == W2) x3 += h2[o];
                if (W3 == 2 * W2) x3 += h2[o < W2 ? o : o - W2];
                g[i] = x3;
              }
            }
            float4* grow = reinterpret_cast<float4*>(sG + tid * P::LDG);
#pragma unroll
            for (int i = 0; i < 4; ++i)
              grow[(c0 / 4 + i) ^ (tid & 7)] = make_float4(g[4 * i], g[4 * i + 1], g[4 * i + 2], g[4 * i + 3]);
          }
          tc::fence_before();
          alive = __syncthreads_and(ok) != 0;
          if (!alive) break;
          // partial xyz of this section: sum_{pairs of the atom} Rn[c] G[n]
          // (FP32, fixed order; plain stores, the atom is owned by this CTA),
          // by accumulator column (rows of N3 columns).  One thread per
          // (atom, 4 columns): per pair one float4 of G and one of Rn feed 16
          // FMAs.
          const int nq = (P::N3 - cb < P::HC ? P::N3 - cb : P::HC) / 4;  // a constant once unrolled
          for (int q = tid; q < ntile * nq; q += blockDim.x) {
            const int k = q / nq, qq = q - k * nq;
            float4 a[4];
#pragma unroll
            for (int c = 0; c < 4; ++c) a[c] = make_float4(0.f, 0.f, 0.f, 0.f);
            for (int pp = s_off[k]; pp < s_off[k + 1]; ++pp) {
              const float4 g = reinterpret_cast<const float4*>(sG + pp * P::LDG)[qq ^ (pp & 7)];
              const float4 r = *reinterpret_cast<const float4*>(sRn + pp * 4);
              const float rc[4] = {r.x, r.y, r.z, r.w};
#pragma unroll
              for (int c = 0; c < 4; ++c) {
                a[c].x = fmaf(rc[c], g.x, a[c].x);
                a[c].y = fmaf(rc[c], g.y, a[c].y);
                a[c].z = fmaf(rc[c], g.z, a[c].z);
                a[c].w = fmaf(rc[c], g.w, a[c].w);
              }
            }
            float4* o = reinterpret_cast<float4*>(xpart + (size_t)s_row[k] * 4 * P::N3 + cb) + qq;
#pragma unroll
            for (int c = 0; c < 4; ++c) o[c * (P::N3 / 4)] = a[c];
          }
          __syncthreads();
        }
      }
    }
    // finalize the chunk, kFinAtoms atoms at a time: xyz = sum over sections
    // / nnei (staged in shared memory), D = xyz^T xyz[:, :axis]
    const float inv = 1.f / (float)p.nnei;
    const int dim = ng * p.axis;
    float* sX = reinterpret_cast<float*>(smem + P::xs);
    for (int r0 = ch.row0; r0 < ch.row1; r0 += kFinAtoms) {
      const int nr = min(kFinAtoms, ch.row1 - r0);
      __syncthreads();
      // (ng == W3: index arithmetic by compile-time divisors only)
      for (int q = tid; q < nr * 4 * W3; q += blockDim.x) {
        const int a = q / (4 * W3), qq = q - a * 4 * W3;
        const int cc = qq / W3, n = qq - cc * W3;
        const int col = cc * P::N3 + neuron_col(n, W3, W2);  // the partials are by accumulator column
        const int r = r0 + a, row = sorted_rows[r];
        float s = 0.f;
        for (int t = 0; t < p.ntypes; ++t)
          if (run_len[(size_t)r * p.ntypes + t] > 0) s += xyzp[((size_t)t * p.nrows + row) * 4 * P::N3 + col];
        s *= inv;
        sX[q] = s;
        xyz[(size_t)row * 4 * W3 + qq] = s;
      }
      __syncthreads();
      // one thread per (atom, neuron n): D[n][m] for every m < axis
      const int M = p.axis;
      for (int q = tid; q < nr * W3; q += blockDim.x) {
        const int a = q / W3, n = q - a * W3;
        const float* xr = sX + a * 4 * W3;
        const float xn[4] = {xr[n], xr[W3 + n], xr[2 * W3 + n], xr[3 * W3 + n]};
        const size_t o = (size_t)(r0 + a) * dim + (size_t)n * M;
        auto dnm = [&](int m) {
          float s = 0.f;
#pragma unroll
          for (int cc = 0; cc < 4; ++cc) s = fmaf(xn[cc], xr[cc * W3 + m], s);
          return s;
        };
        if (e.d_bf16 && M == 16) {  // the tensor-core fitting reads D as BF16: two 16-byte rows
          __nv_bfloat162 h[8];
#pragma unroll
          for (int m = 0; m < 16; m += 2) h[m / 2] = __floats2bfloat162_rn(dnm(m), dnm(m + 1));
          uint4* dst = reinterpret_cast<uint4*>(reinterpret_cast<__nv_bfloat16*>(Dout) + o);
          dst[0] = *reinterpret_cast<const uint4*>(&h[0]);
          dst[1] = *reinterpret_cast<const uint4*>(&h[4]);
        } else if (e.d_bf16) {
          for (int m = 0; m < M; ++m) reinterpret_cast<__nv_bfloat16*>(Dout)[o + m] = __float2bfloat16_rn(dnm(m));
        } else {
          for (int m = 0; m < M; ++m) Dout[o + m] = dnm(m);
        }
      }
    }
    __syncthreads();
  }
  tc::fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tbase, P::tmem_cols);
}

// ---------------------------------------------------------------------------
// Backward of the embedding per tile: forward recompute (t1, t2 kept in
// registers; h1, h2 recomputed from them), then per pair dG = R~ . dxyz,
// dR~ = sum_n G_n dxyz_n, and the chain dP3 -> dH2 -> dP2 -> dH1 -> dR~[0]
// through the two transposed-weight MMAs.  The residual terms of dH2 and dH1
// are folded group by group (col_neuron order) and stored into their
// accumulators before the MMA adds the weight term.
template <int W1, int W2, int W3, bool IDT>
__global__ void __launch_bounds__(128, 3)
emb_tc_bwd_kernel(DescParams<float> p, EmbTC e, const WorkChunk* __restrict__ chunks, int nchunks,
                  const int* __restrict__ run_len, const int* __restrict__ sorted_rows,
                  const float* __restrict__ dxyz, float* __restrict__ gpair, double* __restrict__ vir_row,
                  int* __restrict__ status, int* __restrict__ queue) {
  using P = PlanB<W1, W2, W3>;
  static_assert(W2 == 2 * W1 && W3 == 2 * W2, "the backward folds doubling residuals (w2 = 2 w1, w3 = 2 w2)");
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ uint64_t bar;
  __shared__ uint32_t s_tmem;
  __shared__ int s_row[kTcMaxAtoms], s_off[kTcMaxAtoms + 1], s_ntile, s_cursor;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int ng = p.ng;
  if (warp == 0) tc::tmem_alloc(&s_tmem, P::tmem_cols);
  if (tid == 0) tc::mbar_init(&bar, 1);
  __syncthreads();
  tc::fence_after();
  const uint32_t tbase = s_tmem;
  const uint32_t tlane = tc::taddr(tbase, warp * 32, 0);
  uint32_t phase = 0;
  bool alive = true;
  float* sV = reinterpret_cast<float*>(smem + P::vec);
  float* sVir = reinterpret_cast<float*>(smem + P::vir);
  const uint32_t sA = tc::smem_u32(smem + P::reg);  // A1, A2, dP3, dP2 in turn
  const uint32_t sA1lo = tc::smem_u32(smem + P::a1lo), sA2lo = tc::smem_u32(smem + P::a2lo);
  const uint32_t sW2 = tc::smem_u32(smem + P::fw2), sW3 = tc::smem_u32(smem + P::fw3);
  const uint32_t sB3 = tc::smem_u32(smem + P::bw3), sB2 = tc::smem_u32(smem + P::bw2);
  const float rmin = (float)p.rcut_smth, rmax = (float)p.rcut;
  __shared__ int s_work;
  for (int c = work_first(queue, &s_work); c < nchunks && alive; c = work_next(queue, c, &s_work)) {
    const WorkChunk ch = chunks[c];
    const int ti = ch.ti;
    for (int q = tid; q < (ch.row1 - ch.row0) * 9; q += blockDim.x)
      vir_row[(size_t)sorted_rows[ch.row0 + q / 9] * 9 + q % 9] = 0.0;
    __syncthreads();
    for (int t = 0; t < p.ntypes && alive; ++t) {
      const int net = p.type_one_side ? t : t * p.ntypes + ti;
      copy16(smem + P::fw2, e.fw2 + (size_t)net * P::N2 * P::K1 * 2, P::N2 * P::K1 * 2);
      copy16(smem + P::fw3, e.fw3 + (size_t)net * P::N3 * P::N2 * 2, P::N3 * P::N2 * 2);
      copy16(smem + P::bw3, e.bw3 + (size_t)net * P::N2 * P::N3 * 2, P::N2 * P::N3 * 2);
      copy16(smem + P::bw2, e.bw2 + (size_t)net * P::K1 * P::N2 * 2, P::K1 * P::N2 * 2);
      for (int q = tid; q < P::VEC; q += blockDim.x) sV[q] = e.vec[(size_t)net * P::VEC + q];
      if (tid == 0) s_cursor = ch.row0;
      __syncthreads();
      const float* w1 = sV;
      const float* b1 = sV + P::K1;
      const float* i1 = sV + 2 * P::K1;
      const float* b2 = sV + 3 * P::K1;  // layers 2 and 3: by column (col_neuron order)
      const float* i2 = b2 + P::N2;
      const float* b3 = i2 + P::N2;
      const float* i3 = b3 + P::N3;
      while (alive) {
        if (warp == 0)
          pack_tile<kTcMaxAtoms>(run_len, sorted_rows, p.ntypes, ch.row1, t, s_row, s_off, &s_ntile, &s_cursor,
                                 tid & 31);
        __syncthreads();
        const int ntile = s_ntile;
        if (ntile == 0) break;
        // bring the tile atoms' dE/dxyz rows into L1 now; epilogue 3 reads
        // them after the two forward MMAs
        {
          const int lines = (4 * ng * (int)sizeof(float) + 127) / 128;
          for (int q = tid; q < ntile * lines; q += blockDim.x) {
            const int k = q / lines, l = q - k * lines;
            const char* a = reinterpret_cast<const char*>(dxyz + (size_t)s_row[k] * 4 * ng) + 128 * l;
            asm volatile("prefetch.global.L1 [%0];" ::"l"(a));
          }
        }
        PairInfo pi;
        float rn[4], dv[3];
        pair_env(p, t, ti, s_row, s_off, ntile, tid, pi, rn, dv);
        const float x = rn[0];
        float t1[W1];
#pragma unroll
        for (int k = 0; k < W1; ++k) t1[k] = tanh_fast(fmaf(x, w1[k], b1[k]));
        // h1 = t1 idt1 (+ x when the residual concatenates x); rows past the
        // tile's pairs carry finite values that no output reads
        auto h1 = [&](int k) {
          float h = IDT ? t1[k] * i1[k] : t1[k];
          if (W1 == 1 || W1 == 2) h += x;
          return h;
        };
#pragma unroll
        for (int k0 = 0; k0 < P::K1; k0 += 8) {
          float v[8];
#pragma unroll
          for (int i = 0; i < 8; ++i)
            v[i] = (k0 + i < W1) ? h1(k0 + i) : (k0 + i == P::ONE2a || k0 + i == P::ONE2b ? 1.f : 0.f);
          store8_split(smem + P::a1, smem + P::a1lo, tid, k0, P::K1, v);
        }
        tc::fence_async_smem();
        __syncthreads();
        tc::fence_after();
        if (tid == 0) {
          issue_mma<P::K1, P::N2>(tbase, sA, sW2, P::K1);
          issue_mma<P::K1, P::N2>(tbase, sA1lo, sW2, P::K1, true);
          tc::mma_commit(&bar);
        }
        bool ok = tc::mbar_wait(&bar, phase, status + kStatusTimeout);
        phase ^= 1;
        tc::fence_after();
        // epilogue 2: t2 (neuron order; the accumulator includes b2); A2 = h2 by column
        float t2[W2];
#pragma unroll
        for (int c0 = 0; c0 < P::N2; c0 += 16) {
          float v[16];
          tc::tmem_ld16(tlane + c0, v);
          tc::tmem_ld_wait();
#pragma unroll
          for (int i = 0; i < 16; ++i) {
            const int cc = c0 + i, o = col_neuron(cc, W2, W1);
            if (o >= 0) t2[o] = tanh_fast(v[i]);
          }
        }
        // h2 of neuron o (column cc): t2 idt2 + residual of h1
        auto h2 = [&](int o, int cc) {
          float h = IDT ? t2[o] * i2[cc] : t2[o];
          if (W2 == W1) h += h1(o);
          if (W2 == 2 * W1) h += h1(o < W1 ? o : o - W1);
          return h;
        };
#pragma unroll
        for (int k0 = 0; k0 < P::N2; k0 += 8) {
          float v[8];
#pragma unroll
          for (int i = 0; i < 8; ++i) {
            const int o = col_neuron(k0 + i, W2, W1);
            v[i] = o >= 0 ? h2(o, k0 + i) : (k0 + i == P::ONE3a || k0 + i == P::ONE3b ? 1.f : 0.f);
          }
          store8_split(smem + P::a2, smem + P::a2lo, tid, k0, P::N2, v);
        }
        tc::fence_before();
        tc::fence_async_smem();
        __syncthreads();
        tc::fence_after();
        if (tid == 0) {
          issue_mma<P::N2, P::N3>(tbase, sA, sW3, P::N2);  // over the consumed layer-2 columns
          issue_mma<P::N2, P::N3>(tbase, sA2lo, sW3, P::N2, true);
          tc::mma_commit(&bar);
        }
        ok = tc::mbar_wait(&bar, phase, status + kStatusTimeout) && ok;
        phase ^= 1;
        tc::fence_after();
        // epilogue 3: G, dG = R~ . dxyz, dR~ (direct part), dP3 = dG idt3
        // (1 - t3^2) into the BF16 operand; the residual part of dH2 (dG of
        // both halves folded onto their layer-2 neuron) completes group by
        // group and goes to the dH2 accumulator columns (already read here)
        const float4* dx = reinterpret_cast<const float4*>(dxyz + (size_t)pi.row * 4 * ng);
        float drn[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int c0 = 0; c0 < P::N3; c0 += 16) {
          float v[16], dp[16];
          tc::tmem_ld16(tlane + c0, v);
          tc::tmem_ld_wait();
          // columns i and i + 8: layer-3 neurons o and w2 + o (both feed the
          // residual of layer-2 neuron o, whose dH2 column lies in this group
          // or an earlier one, already read by this lane)
#pragma unroll
          for (int i = 0; i < 8; ++i) {
            float res = 0.f;
#pragma unroll
            for (int h = 0; h < 16; h += 8) {
              const int cc = c0 + i + h, o = col_neuron(cc, W3, W2);
              dp[i + h] = 0.f;
              if (o >= 0) {
                const float tv = tanh_fast(v[i + h]);  // the accumulator includes b3
                const int m = o < W2 ? o : o - W2;
                const float g = (IDT ? tv * i3[cc] : tv) + h2(m, neuron_col(m, W2, W1));
                const float4 dq = pi.valid ? dx[o] : make_float4(0.f, 0.f, 0.f, 0.f);
                drn[0] = fmaf(g, dq.x, drn[0]);
                drn[1] = fmaf(g, dq.y, drn[1]);
                drn[2] = fmaf(g, dq.z, drn[2]);
                drn[3] = fmaf(g, dq.w, drn[3]);
                const float dg = rn[0] * dq.x + rn[1] * dq.y + rn[2] * dq.z + rn[3] * dq.w;
                res += dg;
                dp[i + h] = (IDT ? dg * i3[cc] : dg) * (1.f - tv * tv);
              }
            }
            const int o = col_neuron(c0 + i, W3, W2);
            if (o >= 0) tc::tmem_st1(tlane + neuron_col(o, W2, W1), res);
          }
          store8(smem + P::a3, tid, c0, P::N3, dp);
          store8(smem + P::a3, tid, c0 + 8, P::N3, dp + 8);
        }
        tc::tmem_st_wait();
        tc::fence_before();
        tc::fence_async_smem();
        __syncthreads();
        tc::fence_after();
        if (tid == 0) {
          issue_mma<P::N3, P::N2>(tbase, sA, sB3, P::N3, true);  // dH2 += dP3 . W3^T
          tc::mma_commit(&bar);
        }
        ok = tc::mbar_wait(&bar, phase, status + kStatusTimeout) && ok;
        phase ^= 1;
        tc::fence_after();
        // epilogue 4: dP2 = dH2 idt2 (1 - t2^2) into the operand; the
        // residual of dH1 folds group by group into its accumulator
#pragma unroll
        for (int c0 = 0; c0 < P::N2; c0 += 16) {
          float v[16], dp[16];
          tc::tmem_ld16(tlane + c0, v);
          tc::tmem_ld_wait();
#pragma unroll
          for (int i = 0; i < 16; ++i) {
            const int cc = c0 + i, o = col_neuron(cc, W2, W1);
            dp[i] = o >= 0 ? (IDT ? v[i] * i2[cc] : v[i]) * (1.f - t2[o] * t2[o]) : 0.f;
          }
          store8(smem + P::a2, tid, c0, P::N2, dp);
          store8(smem + P::a2, tid, c0 + 8, P::N2, dp + 8);
          // residual of dH1: layer-1 neurons 8 (c0 / 16) .. + 7, both halves
          // in this group, to their dH1 columns n2 + c0 / 2 ..
          float r[8];
#pragma unroll
          for (int i = 0; i < 8; ++i) r[i] = col_neuron(c0 + i, W2, W1) >= 0 ? v[i] + v[i + 8] : 0.f;
          tc::tmem_st8(tlane + P::N2 + c0 / 2, r);
        }
        tc::tmem_st_wait();
        tc::fence_before();
        tc::fence_async_smem();
        __syncthreads();
        tc::fence_after();
        if (tid == 0) {
          issue_mma<P::N2, P::K1>(tbase + P::N2, sA, sB2, P::N2, true);  // dH1 += dP2 . W2^T
          tc::mma_commit(&bar);
        }
        ok = tc::mbar_wait(&bar, phase, status + kStatusTimeout) && ok;
        phase ^= 1;
        tc::fence_after();
        float dss = 0.f;
#pragma unroll
        for (int c0 = 0; c0 < P::K1; c0 += 16) {
          float v[16];
          tc::tmem_ld16(tlane + P::N2 + c0, v);
          tc::tmem_ld_wait();
#pragma unroll
          for (int i = 0; i < 16; ++i) {
            const int k = c0 + i;
            if (k < W1) {
              const float dh = v[i];
              dss = fmaf((IDT ? dh * i1[k] : dh) * (1.f - t1[k] * t1[k]), w1[k], dss);
              if (W1 == 1 || W1 == 2) dss += dh;
            }
          }
        }
        drn[0] += dss;
        // pair gradient g = dE/d(r_j - r_i) and the pair virial -g (x) d
        float g[3] = {0.f, 0.f, 0.f};
        if (pi.valid && pi.nb >= 0 && pi.keep) {
          float der[12];
          env_deriv(dv, rmin, rmax, der);
          const float* sdi = p.dstd_inv + ((size_t)ti * p.nnei + pi.slot) * 4;
#pragma unroll
          for (int cc = 0; cc < 4; ++cc) {
            const float w = drn[cc] * sdi[cc];
#pragma unroll
            for (int k = 0; k < 3; ++k) g[k] -= w * der[3 * cc + k];
          }
        }
        if (p.facc) {  // -g onto the neighbour's row as 2^-32 fixed point
          if (pi.valid && pi.nb >= 0 && pi.keep) {
            unsigned long long* a = p.facc + 3 * (size_t)neighbour_row(p, pi.row, pi.nb);
#pragma unroll
            for (int k = 0; k < 3; ++k) atomicAdd(a + k, (unsigned long long)__float2ll_rn(-g[k] * kFixScale));
          }
        } else if (pi.valid) {
          float* gp = gpair + ((size_t)pi.row * p.nnei + pi.slot) * 3;
          gp[0] = g[0];
          gp[1] = g[1];
          gp[2] = g[2];
        }
        // the operand region is free (the last MMA completed): pair virials
        // and (fixed-point forces) the pair gradients, 12 per pair
#pragma unroll
        for (int k = 0; k < 3; ++k) {
#pragma unroll
          for (int l = 0; l < 3; ++l) sVir[tid * 12 + 3 * k + l] = -g[k] * dv[l];
          sVir[tid * 12 + 9 + k] = g[k];
        }
        tc::fence_before();
        alive = __syncthreads_and(ok) != 0;
        if (!alive) break;
        const int ncomp = p.facc ? 12 : 9;
        for (int q = tid; q < ntile * ncomp; q += blockDim.x) {
          const int k = q / ncomp, comp = q - ncomp * k;
          float hi = 0.f, lo = 0.f;  // compensated FP32 sum (the FP64 pipe is narrow)
          for (int pp = s_off[k]; pp < s_off[k + 1]; ++pp) comp_add(hi, lo, sVir[pp * 12 + comp]);
          if (comp < 9)
            vir_row[(size_t)s_row[k] * 9 + comp] += (double)hi + (double)lo;
          else  // the atom's own pairs
            atomicAdd(p.facc + 3 * (size_t)s_row[k] + comp - 9,
                      (unsigned long long)llrint(((double)hi + (double)lo) * (double)kFixScale));
        }
        __syncthreads();
      }
    }
  }
  tc::fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tbase, P::tmem_cols);
}

// run lengths of active slots per (sorted row, section)
// one warp per sorted row: the row's slots are read once, coalesced, and
// each type section's count of real neighbours is a warp sum
__global__ void run_len_kernel(int* __restrict__ run_len, const int* __restrict__ nlist,
                               const int* __restrict__ sorted_rows, int nrows, int nnei, SelInfo sel, int pad_zero) {
  const int r = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
  if (r >= nrows) return;  // the whole warp
  const int* nl = nlist + (size_t)sorted_rows[r] * nnei;
  for (int t = 0; t < sel.ntypes; ++t) {
    int n = sel.sel[t];
    if (pad_zero) {
      int c = 0;
      for (int k = sel.sec[t] + lane; k < sel.sec[t] + sel.sel[t]; k += 32) c += nl[k] >= 0;
      n = __reduce_add_sync(0xffffffffu, c);
    }
    if (lane == 0) run_len[(size_t)r * sel.ntypes + t] = n;
  }
}

// dE/dxyz (before the forward's 1/nnei): dxyz[n][c] = (sum_m dD[n][m] xyz[c][m]
// + [n < M] sum_n' dD[n'][n] xyz[c][n']) / nnei, stored [row][ng][4] (one
// float4 per neuron for the backward kernels).  One warp per row, all in
// registers: lane l owns neurons l + 32 k and their M = 16 entries of dD;
// xyz[:, :M] is loaded by every lane (broadcast); the second term's 4 x M
// partial sums are combined across the warp by a reduce-scatter of
// shuffles (five halvings leave T[2l], T[2l+1] in lane l).
constexpr int kDxyzM = 16, kDxyzWarps = 4;

__global__ void __launch_bounds__(kDxyzWarps * 32)
dxyz_kernel(float* __restrict__ dxyz, const float* __restrict__ dD, const float* __restrict__ xyz,
            const int* __restrict__ row_pos, const int* __restrict__ atype, int nloc, int nrows, int ng, int nnei) {
  constexpr int M = kDxyzM;
  const int lane = threadIdx.x & 31;
  const int row = blockIdx.x * kDxyzWarps + (threadIdx.x >> 5);
  if (row >= nrows) return;
  float4* out = reinterpret_cast<float4*>(dxyz + (size_t)row * 4 * ng);
  if (atype[row % nloc] < 0) {
    for (int n = lane; n < ng; n += 32) out[n] = make_float4(0.f, 0.f, 0.f, 0.f);
    return;
  }
  const float* xr = xyz + (size_t)row * 4 * ng;  // [c][n]
  const float* d = dD + (size_t)row_pos[row] * ng * M;  // [n][m]
  float xm[4][M];  // xyz[c][m], m < M
#pragma unroll
  for (int c = 0; c < 4; ++c)
#pragma unroll
    for (int m4 = 0; m4 < M; m4 += 4) {
      const float4 q = *reinterpret_cast<const float4*>(xr + c * ng + m4);
      xm[c][m4] = q.x;
      xm[c][m4 + 1] = q.y;
      xm[c][m4 + 2] = q.z;
      xm[c][m4 + 3] = q.w;
    }
  float T[4 * M];  // partial sum_n' dD[n'][m] xyz[c][n'] over this lane's n', index c * M + m
#pragma unroll
  for (int q = 0; q < 4 * M; ++q) T[q] = 0.f;
  const float inv = 1.f / (float)nnei;
  float4 first = make_float4(0.f, 0.f, 0.f, 0.f);  // term 1 of neuron lane (< M), completed after the reduction
  for (int n = lane; n < ng; n += 32) {
    float dd[M];
    const float4* dq = reinterpret_cast<const float4*>(d + (size_t)n * M);
#pragma unroll
    for (int m4 = 0; m4 < M / 4; ++m4) {
      const float4 q = dq[m4];
      dd[4 * m4] = q.x;
      dd[4 * m4 + 1] = q.y;
      dd[4 * m4 + 2] = q.z;
      dd[4 * m4 + 3] = q.w;
    }
    float t1[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      float s = 0.f;
#pragma unroll
      for (int m = 0; m < M; ++m) s = fmaf(dd[m], xm[c][m], s);
      t1[c] = s;
      const float xn = xr[c * ng + n];
#pragma unroll
      for (int m = 0; m < M; ++m) T[c * M + m] = fmaf(dd[m], xn, T[c * M + m]);
    }
    if (n < M)
      first = make_float4(t1[0], t1[1], t1[2], t1[3]);
    else
      out[n] = make_float4(t1[0] * inv, t1[1] * inv, t1[2] * inv, t1[3] * inv);
  }
  // reduce-scatter of T over the warp: at each halving a lane keeps the half
  // its lane bit selects and adds the partner's copy of it
#pragma unroll
  for (int h = 32, o = 16; h >= 2; h >>= 1, o >>= 1) {
    const bool upper = (lane & o) != 0;
#pragma unroll
    for (int i = 0; i < h; ++i) {
      const float send = upper ? T[i] : T[i + h];
      const float keep = upper ? T[i + h] : T[i];
      T[i] = keep + __shfl_xor_sync(0xffffffffu, send, o);
    }
  }
  // lane l now holds T[2l] and T[2l + 1]; neuron n < M takes T[c * M + n]
  float tc[4];
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    const int q = c * M + (lane & (M - 1));
    const float a0 = __shfl_sync(0xffffffffu, T[0], q >> 1), a1 = __shfl_sync(0xffffffffu, T[1], q >> 1);
    tc[c] = (q & 1) ? a1 : a0;
  }
  if (lane < M && lane < ng)
    out[lane] = make_float4((first.x + tc[0]) * inv, (first.y + tc[1]) * inv, (first.z + tc[2]) * inv,
                            (first.w + tc[3]) * inv);
}

// The same for any axis width: one warp per row with the row's xyz and dD
// staged in shared memory (dD transposed so lanes over n read consecutive
// words).
__global__ void dxyz_smem_kernel(float* __restrict__ dxyz, const float* __restrict__ dD, const float* __restrict__ xyz,
                            const int* __restrict__ row_pos, const int* __restrict__ atype, int nloc, int nrows,
                            int ng, int M, int nnei) {
  extern __shared__ float s_dx[];
  const int wpb = blockDim.x >> 5, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int row = blockIdx.x * wpb + warp;
  if (row >= nrows) return;
  float* sx = s_dx + (size_t)warp * (4 * ng + ng * M + 4 * M);
  float* sdT = sx + 4 * ng;  // dD transposed: [m][n], so lanes over n read consecutive words
  float* sT = sdT + ng * M;  // T[c][m] = sum_n' dD[n'][m] xyz[c][n']
  float* out = dxyz + (size_t)row * 4 * ng;
  if (atype[row % nloc] < 0) {
    for (int q = lane; q < 4 * ng; q += 32) out[q] = 0.f;
    return;
  }
  const float* xr = xyz + (size_t)row * 4 * ng;
  const float* d = dD + (size_t)row_pos[row] * ng * M;
  for (int q = lane; q < 4 * ng; q += 32) sx[q] = xr[q];
  for (int q = lane; q < ng * M; q += 32) {
    const int n = q / M, m = q - n * M;
    sdT[m * ng + n] = d[q];
  }
  __syncwarp();
  for (int q = lane; q < 4 * M; q += 32) {
    const int c = q / M, m = q - c * M;
    const float* xc = sx + c * ng;
    const float* dm = sdT + m * ng;
    float s = 0.f;
    for (int n2 = 0; n2 < ng; ++n2) s = fmaf(dm[n2], xc[n2], s);
    sT[q] = s;
  }
  __syncwarp();
  const float inv = 1.f / (float)nnei;
  for (int q = lane; q < 4 * ng; q += 32) {  // out [n][c]: one float4 per neuron
    const int n = q >> 2, c = q & 3;
    const float* xc = sx + c * ng;
    float s = n < M ? sT[c * M + n] : 0.f;
    for (int m = 0; m < M; ++m) s = fmaf(sdT[m * ng + n], xc[m], s);
    out[q] = s * inv;
  }
}

template <int W1, int W2, int W3, bool IDT>
int launch_fwd_t(const DescParams<float>& p, const EmbTC& e, const WorkChunk* chunks, int nchunks, const int* run_len,
                 const int* sorted_rows, float* xyz, float* xyzp, float* D, int* status, cudaStream_t st, int nsm,
                 int* queue) {
  using P = PlanF<W1, W2, W3>;
  auto k = emb_tc_fwd_kernel<W1, W2, W3, IDT>;
  DPGB_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, P::total));
  const int grid = nchunks < nsm ? nchunks : nsm;
  k<<<grid, 128, P::total, st>>>(p, e, chunks, nchunks, run_len, sorted_rows, xyz, xyzp, D, status, queue);
  return check_launch("emb_tc_fwd");
}
template <int W1, int W2, int W3, bool IDT>
int launch_bwd_t(const DescParams<float>& p, const EmbTC& e, const WorkChunk* chunks, int nchunks, const int* run_len,
                 const int* sorted_rows, const float* dxyz, float* gpair, double* vir_row, int* status, cudaStream_t st,
                 int nsm, int* queue) {
  using P = PlanB<W1, W2, W3>;
  auto k = emb_tc_bwd_kernel<W1, W2, W3, IDT>;
  DPGB_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, P::total));
  const int grid = nchunks < nsm ? nchunks : nsm;
  k<<<grid, 128, P::total, st>>>(p, e, chunks, nchunks, run_len, sorted_rows, dxyz, gpair, vir_row, status, queue);
  return check_launch("emb_tc_bwd");
}


}  // namespace

int launch_run_lengths(int* run_len, const int* nlist, const int* sorted_rows, int nrows, int nnei, const SelInfo& sel,
                       int pad_zero, cudaStream_t st) {
  if (nrows <= 0) return DPGB_OK;
  run_len_kernel<<<ceil_div(nrows, 8), 256, 0, st>>>(run_len, nlist, sorted_rows, nrows, nnei, sel, pad_zero);
  return check_launch("run_len");
}

int launch_emb_tc_fwd(const DescParams<float>& p, const EmbTC& e, const WorkChunk* chunks, int nchunks,
                      const int* run_len, const int* sorted_rows, float* xyz, float* xyzp, float* D, int* status,
                      cudaStream_t st, int* queue) {
  if (nchunks <= 0) return DPGB_OK;
  const int nsm = 3 * sm_count();  // three CTAs per SM
  const bool idt = e.has_idt1 || e.has_idt2 || e.has_idt3;
#define DPGB_FWD(a, b, c, i) \
  launch_fwd_t<a, b, c, i>(p, e, chunks, nchunks, run_len, sorted_rows, xyz, xyzp, D, status, st, nsm, queue)
  if (e.w1 == 25 && e.w2 == 50 && e.w3 == 100) return idt ? DPGB_FWD(25, 50, 100, true) : DPGB_FWD(25, 50, 100, false);
  if (e.w1 == 3 && e.w2 == 6 && e.w3 == 12) return idt ? DPGB_FWD(3, 6, 12, true) : DPGB_FWD(3, 6, 12, false);
#undef DPGB_FWD
  return fail(DPGB_EINVAL, "embedding widths without a tensor-core kernel");
}

int launch_dxyz(const DescParams<float>& p, const float* dD, const float* xyz, float* dxyz, cudaStream_t st) {
  if (p.nrows <= 0) return DPGB_OK;
  if (p.axis == kDxyzM && p.ng % 4 == 0) {
    dxyz_kernel<<<ceil_div(p.nrows, kDxyzWarps), kDxyzWarps * 32, 0, st>>>(dxyz, dD, xyz, p.row_pos, p.atype,
                                                                          p.nloc, p.nrows, p.ng, p.nnei);
    return check_launch("dxyz");
  }
  const int ng = p.ng, M = p.axis;
  const size_t per_warp = sizeof(float) * (4 * ng + ng * M + 4 * M);
  int wpb = 8;
  while (wpb > 1 && per_warp * wpb > 96 * 1024) wpb >>= 1;
  DPGB_CUDA(cudaFuncSetAttribute(dxyz_smem_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(per_warp * wpb)));
  dxyz_smem_kernel<<<ceil_div(p.nrows, wpb), 32 * wpb, per_warp * wpb, st>>>(dxyz, dD, xyz, p.row_pos, p.atype,
                                                                             p.nloc, p.nrows, ng, M, p.nnei);
  return check_launch("dxyz");
}

int launch_emb_tc_bwd(const DescParams<float>& p, const EmbTC& e, const WorkChunk* chunks, int nchunks,
                      const int* run_len, const int* sorted_rows, const float* dxyz, float* gpair, double* vir_row,
                      int* status, cudaStream_t st, int* queue) {
  if (nchunks <= 0) return DPGB_OK;
  const int nsm = 3 * sm_count();  // three CTAs per SM
  const bool idt = e.has_idt1 || e.has_idt2 || e.has_idt3;
#define DPGB_BWD(a, b, c, i) \
  launch_bwd_t<a, b, c, i>(p, e, chunks, nchunks, run_len, sorted_rows, dxyz, gpair, vir_row, status, st, nsm, queue)
  if (e.w1 == 25 && e.w2 == 50 && e.w3 == 100) return idt ? DPGB_BWD(25, 50, 100, true) : DPGB_BWD(25, 50, 100, false);
  if (e.w1 == 3 && e.w2 == 6 && e.w3 == 12) return idt ? DPGB_BWD(3, 6, 12, true) : DPGB_BWD(3, 6, 12, false);
#undef DPGB_BWD
  return fail(DPGB_EINVAL, "embedding widths without a tensor-core kernel");
}

}  // namespace dpgb
