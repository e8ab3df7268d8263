// DeepPot: the se_e2_a energy / force / virial evaluation behind the C API
// (source/api_c/include/c_api.h:150,244-322, source/api_cc/src/DeepPotPT.cc:
// 170-378 semantics: wrap, ghost images, typed neighbour list, descriptor,
// fitting, dE/dr, ghost-to-local force reduction, virial).
//
// Pipeline per call (all on one stream, no host synchronisation in the
// device form):
//   normalise -> cell-list neighbour list (per frame) -> sorted transpose of
//   the list -> desc_fwd -> fitting fwd+bwd per type -> desc_bwd ->
//   force / atomic-virial gather -> per-frame FP64 energy and virial sums.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <memory>
#include <numeric>
#include <string>
#include <vector>

#include <type_traits>

#include "emb_tc.cuh"
#include "fit_tc.cuh"
#include "se_a.cuh"

namespace dpgb {
namespace {

template <typename T>
struct DevModel {
  EmbParams<T> emb{};
  FitParams<T> fit{};
  T* davg = nullptr;
  T* dstd = nullptr;
  T* dstd_inv = nullptr;
  TabMeta<T>* meta = nullptr;
  std::vector<DeviceBuffer*> owned;
  ~DevModel() {
    for (auto* b : owned) delete b;
  }
  template <typename S>
  T* upload(const std::vector<S>& h) {
    std::vector<T> c(h.begin(), h.end());
    auto* b = new DeviceBuffer();
    owned.push_back(b);
    if (b->alloc(sizeof(T) * std::max<size_t>(c.size(), 1)) != DPGB_OK) return nullptr;
    if (!c.empty() && cudaMemcpy(b->ptr, c.data(), sizeof(T) * c.size(), cudaMemcpyHostToDevice) != cudaSuccess)
      return nullptr;
    return b->as<T>();
  }
};

// ---- pipeline kernels --------------------------------------------------------
__global__ void model_keys_kernel(int* __restrict__ keys, const int* __restrict__ nlist, int npair, FastDiv by_nnei,
                                  int nloc, FastDiv by_nloc) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npair) return;
  const int nb = nlist[p];
  const int f = by_nloc.div(by_nnei.div(p));
  keys[p] = nb < 0 ? -1 : f * nloc + (nb - by_nloc.div(nb) * nloc);
}

// F[row] = sum_slots g[row] - sum_{pairs -> row} g;  optional atomic virial on
// the neighbour: -sum_{pairs -> row} g (x) d.  One warp per atom: lanes take
// the atom's slots and its transposed pairs in a fixed interleave (partial
// sums in GatherAcc), then a fixed xor-shuffle tree (identical in every
// lane), so the result is the same on every run.
constexpr int kGatherWarps = 4;

// Force accumulators of the gathers.  FP64 gradients add in FP64.  FP32
// gradients add in FP32 as an unevaluated sum hi + lo kept exact by the
// two-sum transformation (Knuth), which is as accurate as FP64 accumulation
// of FP32 terms here and stays off the (narrow) FP64 pipe.
template <typename T>
struct GatherAcc {
  double v[3] = {0.0, 0.0, 0.0};
  __device__ __forceinline__ void add(int c, T x) { v[c] += (double)x; }
  __device__ __forceinline__ void reduce() {
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v[c] += __shfl_xor_sync(0xffffffffu, v[c], o);
  }
  __device__ __forceinline__ double get(int c) const { return v[c]; }
};

template <>
struct GatherAcc<float> {
  float hi[3] = {0.f, 0.f, 0.f}, lo[3] = {0.f, 0.f, 0.f};
  __device__ __forceinline__ void add(int c, float x) { comp_add(hi[c], lo[c], x); }
  __device__ __forceinline__ void reduce() {
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const float oh = __shfl_xor_sync(0xffffffffu, hi[c], o), ol = __shfl_xor_sync(0xffffffffu, lo[c], o);
        float e;
        two_sum(hi[c], oh, hi[c], e);
        lo[c] += ol + e;
      }
  }
  __device__ __forceinline__ double get(int c) const { return (double)hi[c] + (double)lo[c]; }
};

// the atom's own slots
template <typename T>
__device__ __forceinline__ void gather_own_slots(GatherAcc<T>& f, const T* __restrict__ gr,
                                                 const int* __restrict__ nr, int nnei, int lane) {
  for (int s = lane; s < nnei; s += 32) {
    if (nr[s] < 0) continue;  // padding slots carry no force (and may be unwritten)
#pragma unroll
    for (int c = 0; c < 3; ++c) f.add(c, gr[3 * s + c]);
  }
}

// the transposed pairs of an atom (pairs whose neighbour it is), four per
// lane at a time: the pair ids first, then their gradients, so that each
// lane keeps several independent gathers in flight
template <typename T, bool AV, typename Disp>
__device__ __forceinline__ void gather_transposed(GatherAcc<T>& f, double av[9], const T* __restrict__ g,
                                                  const Transpose& tr, int a, int lane, Disp disp) {
  const int t1 = tr.offsets[a + 1];
  for (int base = tr.offsets[a]; base < t1; base += 128) {
    int pp[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int t = base + lane + 32 * k;
      pp[k] = t < t1 ? tr.pairs[t] : -1;
    }
    T gv[4][3];
#pragma unroll
    for (int k = 0; k < 4; ++k)
#pragma unroll
      for (int c = 0; c < 3; ++c) gv[k][c] = pp[k] >= 0 ? g[3 * (size_t)pp[k] + c] : T(0);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      if (pp[k] < 0) continue;
#pragma unroll
      for (int c = 0; c < 3; ++c) f.add(c, -gv[k][c]);
      if (AV) {
        double d[3];
        disp(pp[k], d);
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int l = 0; l < 3; ++l) av[3 * i + l] -= (double)gv[k][i] * d[l];
      }
    }
  }
}

template <typename T, bool AV>
__device__ __forceinline__ void gather_store(double* __restrict__ force, double* __restrict__ atom_vir, size_t a,
                                             GatherAcc<T>& f, double av[9], int lane) {
  f.reduce();
  if (AV)
#pragma unroll
    for (int k = 0; k < 9; ++k)
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) av[k] += __shfl_xor_sync(0xffffffffu, av[k], o);
  if (lane == 0) {
#pragma unroll
    for (int c = 0; c < 3; ++c) force[3 * a + c] = f.get(c);
    if (AV)
#pragma unroll
      for (int k = 0; k < 9; ++k) atom_vir[9 * a + k] = av[k];
  }
}

template <typename T, bool AV>
__global__ void __launch_bounds__(kGatherWarps * 32)
force_gather_model_kernel(double* __restrict__ force, double* __restrict__ atom_vir, const T* __restrict__ g,
                          Transpose tr, const int* __restrict__ nlist, const double* __restrict__ coord,
                          const double* __restrict__ svec, int nshift, int nloc, int nnei, int nrows) {
  const int lane = threadIdx.x & 31;
  const int row = blockIdx.x * kGatherWarps + (threadIdx.x >> 5);
  if (row >= nrows) return;
  GatherAcc<T> f;
  gather_own_slots(f, g + (size_t)row * nnei * 3, nlist + (size_t)row * nnei, nnei, lane);
  double av[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) av[k] = 0.0;
  gather_transposed<T, AV>(f, av, g, tr, row, lane, [&](int p, double d[3]) {
    const int prow = p / nnei;
    const int fr = prow / nloc, i = prow - fr * nloc;
    const int nb = nlist[p];
    const int s = nb / nloc, jj = nb - s * nloc;
    const double* cf = coord + (size_t)fr * nloc * 3;
    const double* sv = svec + ((size_t)fr * nshift + s) * 3;
    d[0] = (cf[3 * jj] + sv[0]) - cf[3 * i];
    d[1] = (cf[3 * jj + 1] + sv[1]) - cf[3 * i + 1];
    d[2] = (cf[3 * jj + 2] + sv[2]) - cf[3 * i + 2];
  });
  gather_store<T, AV>(force, atom_vir, (size_t)row, f, av, lane);
}

// Mixed form without atomic virials: the forces of a local model list with
// no transpose.  A row's pair gradients g add up in a fixed order (as in
// force_gather_model_kernel); that sum, and each pair's share on its
// neighbour, -g, are scaled by 2^32, rounded to integers and added with
// 64-bit integer atomics (red) into acc — integer sums are exact, so the
// result does not depend on the order of the adds and repeats bitwise (the
// rounding: 2^-33 per term, far below FP32 resolution at the force scale).
// The table backward does the same inline (DescParams::facc);
// force_fix_kernel then converts acc to the forces.

__global__ void __launch_bounds__(kGatherWarps * 32)
force_scatter_model_kernel(unsigned long long* __restrict__ acc,
                           const float* __restrict__ g, const int* __restrict__ nlist, int nloc, FastDiv by_nloc,
                           int nnei, int nrows) {
  const int lane = threadIdx.x & 31;
  const int row = blockIdx.x * kGatherWarps + (threadIdx.x >> 5);
  if (row >= nrows) return;
  const int fbase = by_nloc.div(row) * nloc;  // the frame's first row
  const float* gr = g + (size_t)row * nnei * 3;
  const int* nr = nlist + (size_t)row * nnei;
  GatherAcc<float> f;
  for (int s = lane; s < nnei; s += 32) {
    const int nb = nr[s];
    if (nb < 0) continue;  // padding slots carry no force (and may be unwritten)
    unsigned long long* a = acc + 3 * (size_t)(fbase + nb - by_nloc.div(nb) * nloc);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float x = gr[3 * s + c];
      f.add(c, x);
      atomicAdd(a + c, (unsigned long long)__float2ll_rn(-x * kFixScale));
    }
  }
  f.reduce();
  if (lane == 0)
#pragma unroll
    for (int c = 0; c < 3; ++c)
      atomicAdd(acc + 3 * (size_t)row + c, (unsigned long long)llrint(f.get(c) * (double)kFixScale));
}

__global__ void force_fix_kernel(double* __restrict__ force, const unsigned long long* __restrict__ acc, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) force[i] = (double)(long long)acc[i] * (1.0 / 4294967296.0);
}

// The same with explicit extended atoms (external list, one frame): every one
// of the nall atoms gets its force and atomic virial (the caller sums ghost
// entries back onto their owners, as LAMMPS's reverse communication does).
template <typename T, bool AV>
__global__ void __launch_bounds__(kGatherWarps * 32)
force_gather_ext_kernel(double* __restrict__ force, double* __restrict__ atom_vir, const T* __restrict__ g,
                        Transpose tr, const int* __restrict__ nlist, const double* __restrict__ coord_ext, int nloc,
                        int nall, int nnei) {
  const int lane = threadIdx.x & 31;
  const int e = blockIdx.x * kGatherWarps + (threadIdx.x >> 5);
  if (e >= nall) return;
  GatherAcc<T> f;
  if (e < nloc) gather_own_slots(f, g + (size_t)e * nnei * 3, nlist + (size_t)e * nnei, nnei, lane);
  double av[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) av[k] = 0.0;
  gather_transposed<T, AV>(f, av, g, tr, e, lane, [&](int p, double d[3]) {
    const int i = p / nnei;
#pragma unroll
    for (int l = 0; l < 3; ++l) d[l] = coord_ext[3 * e + l] - coord_ext[3 * i + l];
  });
  gather_store<T, AV>(force, atom_vir, (size_t)e, f, av, lane);
}

// batch of frames: the key of a pair is its neighbour's global atom
__global__ void batch_keys_kernel(int* __restrict__ keys, const int* __restrict__ nlist, long long npair, int nnei,
                                  FrameTab ft) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npair) return;
  const int nb = nlist[p];
  if (nb < 0) {
    keys[p] = -1;
    return;
  }
  const int row = (int)(p / nnei);
  const int fr = frame_of(ft.atom_off, ft.nframes, row);
  const int beg = ft.atom_off[fr], nl = ft.atom_off[fr + 1] - beg;
  keys[p] = beg + nb % nl;
}

// force_gather_model_kernel for a batch (per-frame image shifts)
template <typename T, bool AV>
__global__ void __launch_bounds__(kGatherWarps * 32)
force_gather_batch_kernel(double* __restrict__ force, double* __restrict__ atom_vir, const T* __restrict__ g,
                          Transpose tr, const int* __restrict__ nlist, const double* __restrict__ coord,
                          const double* __restrict__ svec, FrameTab ft, int nnei, int nrows) {
  const int lane = threadIdx.x & 31;
  const int row = blockIdx.x * kGatherWarps + (threadIdx.x >> 5);
  if (row >= nrows) return;
  GatherAcc<T> f;
  gather_own_slots(f, g + (size_t)row * nnei * 3, nlist + (size_t)row * nnei, nnei, lane);
  double av[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) av[k] = 0.0;
  gather_transposed<T, AV>(f, av, g, tr, row, lane, [&](int p, double d[3]) {
    const int i = p / nnei;  // centre (global row)
    const int fr = frame_of(ft.atom_off, ft.nframes, i);
    const int beg = ft.atom_off[fr], nl = ft.atom_off[fr + 1] - beg;
    const int nb = nlist[p];
    const int s = nb / nl, jj = beg + (nb - s * nl);
    const double* sv = svec + 3 * ((size_t)ft.svec_off[fr] + s);
#pragma unroll
    for (int l = 0; l < 3; ++l) d[l] = (coord[3 * jj + l] + sv[l]) - coord[3 * i + l];
  });
  gather_store<T, AV>(force, atom_vir, (size_t)row, f, av, lane);
}

// Per-frame sums of the atom energies and atom virials in two passes with a
// fixed partition, so the result does not depend on scheduling: pass 1 gives
// every chunk of `chunk` rows of a frame its 10 partial sums (energy, 9
// virial components), pass 2 adds a frame's chunk partials in chunk order.
// Frame f covers rows [atom_off[f], atom_off[f+1]) or, without atom_off,
// [f*nloc, (f+1)*nloc).
constexpr int kFrameSumThreads = 256;

// rows per partial sum: about two blocks per SM over all frames, a power of
// two in [256, 2048]; batches of frames of different sizes keep 2048 (their
// grid spans the largest frame)
int frame_chunk(long long rows, bool batch) {
  if (batch) return 2048;
  const long long want = rows / (2LL * sm_count());
  int c = 256;
  while (c < 2048 && c < want) c <<= 1;
  return c;
}

__global__ void __launch_bounds__(kFrameSumThreads) frame_part_kernel(double* __restrict__ part,
                                                                      const double* __restrict__ e_row,
                                                                      const double* __restrict__ vir_row,
                                                                      const int* __restrict__ atom_off, int nloc,
                                                                      int chunk) {
  const int c = blockIdx.x, f = blockIdx.y, t = threadIdx.x;
  const int lo = atom_off ? atom_off[f] : f * nloc, hi = atom_off ? atom_off[f + 1] : (f + 1) * nloc;
  const int r0 = lo + c * chunk, r1 = min(hi, r0 + chunk);
  double acc[10];
#pragma unroll
  for (int q = 0; q < 10; ++q) acc[q] = 0.0;
  for (int r = r0 + t; r < r1; r += kFrameSumThreads) {
    acc[0] += e_row[r];
#pragma unroll
    for (int q = 0; q < 9; ++q) acc[q + 1] += vir_row[(size_t)r * 9 + q];
  }
  __shared__ double s[kFrameSumThreads / 32][10];
#pragma unroll
  for (int q = 0; q < 10; ++q)
    for (int o = 16; o > 0; o >>= 1) acc[q] += __shfl_down_sync(0xffffffffu, acc[q], o);
  if ((t & 31) == 0)
#pragma unroll
    for (int q = 0; q < 10; ++q) s[t >> 5][q] = acc[q];
  __syncthreads();
  if (t < 10) {
    double v = 0.0;
#pragma unroll
    for (int w = 0; w < kFrameSumThreads / 32; ++w) v += s[w][t];
    part[((size_t)f * gridDim.x + c) * 10 + t] = v;
  }
}

// pass 2: one warp per frame; lane l adds the partials (all 10 sums at
// once) of chunks l, l + 32, ..., then a fixed xor-shuffle tree adds the
// lanes (the same order on every run)
__global__ void frame_final_kernel(double* __restrict__ energy, double* __restrict__ virial,
                                   const double* __restrict__ part, int nchunk, int nframes) {
  const int f = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (f >= nframes) return;  // the whole warp
  double v[10];
#pragma unroll
  for (int q = 0; q < 10; ++q) v[q] = 0.0;
  for (int c = lane; c < nchunk; c += 32) {
    const double* pc = part + ((size_t)f * nchunk + c) * 10;
#pragma unroll
    for (int q = 0; q < 10; ++q) v[q] += pc[q];
  }
#pragma unroll
  for (int q = 0; q < 10; ++q)
    for (int o = 16; o > 0; o >>= 1) v[q] += __shfl_xor_sync(0xffffffffu, v[q], o);
  if (lane == 0) {
    energy[f] = v[0];
#pragma unroll
    for (int q = 1; q < 10; ++q) virial[(size_t)f * 9 + q - 1] = v[q];
  }
}

// FP32 split x = hi + lo of n points (FP64 xyz), for FP32 displacements
__global__ void split_points_kernel(float4* __restrict__ hi, float4* __restrict__ lo, const double* __restrict__ x,
                                   int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float h[3], l[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const double v = x[3 * (size_t)i + k];
    h[k] = (float)v;
    l[k] = (float)(v - (double)h[k]);
  }
  hi[i] = make_float4(h[0], h[1], h[2], 0.f);
  lo[i] = make_float4(l[0], l[1], l[2], 0.f);
}

// atom energy in the original order (+ per-type bias), 0 for virtual atoms
__global__ void atom_energy_kernel(double* __restrict__ e_row, const double* __restrict__ e_sorted,
                                   const int* __restrict__ row_pos, const int* __restrict__ atype,
                                   const double* __restrict__ bias, int nloc, int nrows) {
  const int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= nrows) return;
  const int t = atype[row % nloc];
  e_row[row] = t < 0 ? 0.0 : e_sorted[row_pos[row]] + bias[t];
}

}  // namespace

struct DeepPotImpl {
  dpgb_se_a_desc desc;
  int precision = DPGB_PREC_FP64;
  SelInfo sel{};
  int ng = 0, dim = 0, nnets = 0, pad_zero = 1;
  std::unique_ptr<DevModel<double>> m64;
  std::unique_ptr<DevModel<float>> m32;
  DeviceBuffer bias_dev, pair_mask_dev;
  // host-side caches
  std::vector<int> atype_cache;
  std::vector<int> row_pos_h, type_count, type_off;
  int cached_nframes = -1;
  // bumped whenever cached device state may change (types, workspace): a
  // batch's captured CUDA graph is replayed only while this stays put
  unsigned long long gen = 0;
  DeviceBuffer row_pos_dev, atype_dev, sorted_rows_dev, chunks_dev;
  int nchunks = 0;
  // work queue of the persistent embedding / table kernels (two counters:
  // forward, backward), used when a batch's per-bucket tile sizes cut the
  // work items; the plan the cached rows and items were built for
  DeviceBuffer queue_dev;
  int use_queue = 0;
  const void* plan_owner = nullptr;
  unsigned long long plan_version = 0;
  // tensor-core embedding (mixed precision)
  int use_tc = 0;
  int use_tab = 0;  // compressed nets in the mixed form: fused FP32 table kernels
  EmbTC tc{};
  DeviceBuffer tc_images, tc_vec, ws_runlen, ws_dxyz;
  // tensor-core fitting (mixed precision)
  int use_fit_tc = 0;
  int fit_nh = 0, fit_width[kMaxFitLayers + 1] = {};
  const __nv_bfloat16* fit_Wt[kMaxFitLayers] = {};  // forward B: [nt][out][in]
  const __nv_bfloat16* fit_Wb[kMaxFitLayers] = {};  // backward B: [nt][in][out]
  const float* fit_b[kMaxFitLayers] = {};
  const float* fit_idt[kMaxFitLayers] = {};
  const float* fit_wout = nullptr;
  std::vector<float> fit_bout;
  DeviceBuffer fit_w16, fit_f32, ws_fitb;
  // workspace
  DeviceBuffer ws_nlist, ws_cell, ws_tr, ws_keys, ws_status, ws_coord, ws_svec, ws_spos;
  DeviceBuffer ws_facc;  // fixed-point force sums of the scatter path
  DeviceBuffer ws_D, ws_dD, ws_xyz, ws_g, ws_vir, ws_erow, ws_esorted, ws_act, ws_gbuf, ws_part, ws_xhi, ws_xlo, ws_shi, ws_slo;
  DeviceBuffer ws_env;  // the table path's per-pair environment, forward -> backward
  DeviceBuffer io_coord, io_force, io_av, io_e, io_v, io_ae;
  DeviceBuffer io_out;   // host API: [energy | virial | force | atom energy | atom virial]
  PinnedBuffer io_host;  // host API staging: [coord | the outputs | status words]
  // external neighbour list (CSR over local atoms) kept between calls for
  // `ago` > 0, with the ghost-inclusive types
  DeviceBuffer ext_off, ext_idx, ext_atype;
  int ext_nloc = -1, ext_nall = -1, ext_sorted = 0;
  std::vector<int> ext_atype_h;
  // skin lists (periodic frames; skin 0 = a fresh list every call): the
  // candidates within rcut + skin are rebuilt every `skin_every` calls or when
  // an atom moved more than skin / 2; skin_sel describes the flat candidate
  // rows (width: skin_factor x the count a uniform density gives)
  double skin = 0.0;
  int skin_every = 1;
  int skin_grow = 0;  // > 0: a candidate row needed this many slots: widen, rebuild
  double skin_factor = 1.25;
  SelInfo skin_sel{};
  std::vector<double> skin_box;
  std::vector<int> skin_atype;
  int skin_nframes = -1;
  const void* skin_cand_ptr = nullptr;
  DeviceBuffer ws_gate, ws_cand, ws_skin_off, ws_skin_ref, ws_coordf, ws_svecf, ws_coordflo, ws_svecflo;
  // single-system CUDA graph (dpgb_deeppot_set_graph): one evaluation of a
  // periodic system captured and replayed on the handle's stream while the
  // key (frames, atoms, box, buffers) and the handle's state (gen) hold
  int use_graph = 0;
  int capturing = 0;  // inside a capture: no pageable host uploads (their data is on the device)
  cudaGraph_t sg_graph = nullptr;
  cudaGraphExec_t sg_exec = nullptr;
  unsigned long long sg_gen = ~0ull;
  int sg_nframes = -1, sg_natom = -1, sg_launches = 0;
  // shape of the last single-system evaluation's own neighbour list
  // (ws_nlist, ws_coord, ws_svec), for dpgb_deeppot_last_nlist; 0 frames
  // after an external list or a batch
  int nl_nframes = 0, nl_natom = 0, nl_nshift = 0;
  std::vector<double> sg_box;
  const void* sg_ptr[6] = {};
  cudaEvent_t sg_ev_in = nullptr, sg_ev_out = nullptr;
  // completion of the last evaluation on the caller's stream (the device
  // forms run there, not on `stream`): the status check and the list read
  // without a stream of their own wait for it
  cudaEvent_t last_done = nullptr;
  // descriptor stage on its own (dpgb_deeppot_descrpt_fwd / _bwd): the
  // forward's parameters and extended layout, kept for its backward
  DescParams<float> dm_p{};
  int dm_nf = 0, dm_nloc = 0, dm_nall = 0;
  unsigned long long evals = 0;    // evaluations and descriptor forwards issued (they share the workspace)
  unsigned long long dm_eval = 0;  // the descriptor forward's number; 0: none
  DeviceBuffer dm_keys, dm_tr;
  // side stream of the sorted transpose (needed only by the force gather, so
  // it runs next to the descriptor and the fitting), fork / join events
  cudaStream_t side = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  void drop_graph() {
    if (sg_exec) cudaGraphExecDestroy(sg_exec);
    if (sg_graph) cudaGraphDestroy(sg_graph);
    sg_exec = nullptr;
    sg_graph = nullptr;
    sg_gen = ~0ull;
  }
  std::string err;
  int launches = 0;
  cudaStream_t stream = nullptr;
  // stage timing (events recorded on the compute stream when enabled)
  int profiling = 0;
  cudaEvent_t ev[2 * DPGB_NUM_STAGES] = {};
  int ev_recorded = 0;
  double stage_ms[DPGB_NUM_STAGES] = {};
  int stage_calls = 0;
  void mark(int stage, int end, cudaStream_t st) {
    if (!profiling) return;
    cudaEventRecord(ev[2 * stage + end], st);
    ev_recorded = 1;
  }
};

namespace {

inline int pad64(int k) { return (k + 63) / 64 * 64; }

// host memory the CUDA driver has page-locked (cudaHostAlloc / cudaHostRegister)
bool is_pinned(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();  // clear the sticky-free error of an unknown pointer
    return false;
  }
  return a.type == cudaMemoryTypeHost;
}

// host inputs: every coordinate (and cell entry) must be finite
int check_finite(const double* x, size_t n, const char* what) {
  for (size_t i = 0; i < n; ++i)
    if (!std::isfinite(x[i]))
      return fail(DPGB_EINVAL, std::string("non-finite ") + what + " (entry " + std::to_string(i) + ")");
  return DPGB_OK;
}

// split-BF16 row of a weight image: the high parts of w[0 .. K) in columns
// [0, K), their low parts (the BF16 rounding of w - hi) in [Kp, Kp + K),
// zeros elsewhere
template <typename F>
void push_split_row(std::vector<__nv_bfloat16>& img, int K, int Kp, F w) {
  const size_t b = img.size();
  img.resize(b + 2 * (size_t)Kp, __float2bfloat16_rn(0.f));
  for (int k = 0; k < K; ++k) {
    const double v = w(k);
    const __nv_bfloat16 hi = __float2bfloat16_rn((float)v);
    img[b + k] = hi;
    img[b + Kp + k] = __float2bfloat16_rn((float)(v - (double)__bfloat162float(hi)));
  }
}

// split-BF16 weight images of the tensor-core fitting: forward B = W^T
// [out][hi | lo of in], backward B = W [in][hi | lo of out] per type (rows
// padded to whole 64-column chunks per part); FP32 bias / timestep / output
// layer.
int build_fit_tc(DeepPotImpl& im, const dpgb_se_a_desc& d) {
  const int nt = d.ntypes;
  im.fit_nh = d.n_fit;
  im.fit_width[0] = d.dim_descrpt;
  for (int l = 0; l < d.n_fit; ++l) im.fit_width[l + 1] = d.fit_neuron[l];
  std::vector<__nv_bfloat16> w16;
  std::vector<float> f32;
  size_t offWt[kMaxFitLayers], offWb[kMaxFitLayers], offb[kMaxFitLayers], offi[kMaxFitLayers];
  for (int l = 0; l < d.n_fit; ++l) {
    const int a = im.fit_width[l], o = im.fit_width[l + 1];
    const double* W = d.fit_w[0][l];
    offWt[l] = w16.size();
    for (int t = 0; t < nt; ++t) {
      W = d.fit_w[t][l];
      for (int n = 0; n < o; ++n) push_split_row(w16, a, pad64(a), [&](int k) { return W[(size_t)k * o + n]; });
    }
    offWb[l] = w16.size();
    for (int t = 0; t < nt; ++t) {
      W = d.fit_w[t][l];
      for (int k = 0; k < a; ++k) push_split_row(w16, o, pad64(o), [&](int n) { return W[(size_t)k * o + n]; });
    }
    offb[l] = f32.size();
    for (int t = 0; t < nt; ++t)
      for (int n = 0; n < o; ++n) f32.push_back((float)d.fit_b[t][l][n]);
    offi[l] = (size_t)-1;
    bool has = false;
    for (int t = 0; t < nt; ++t) has |= d.fit_idt[t][l] != nullptr;
    if (has) {
      offi[l] = f32.size();
      for (int t = 0; t < nt; ++t)
        for (int n = 0; n < o; ++n) f32.push_back(d.fit_idt[t][l] ? (float)d.fit_idt[t][l][n] : 1.f);
    }
  }
  const int wl = im.fit_width[d.n_fit];
  const size_t offw = f32.size();
  im.fit_bout.assign(nt, 0.f);
  for (int t = 0; t < nt; ++t) {
    for (int n = 0; n < wl; ++n) f32.push_back((float)d.fit_w[t][d.n_fit][n]);
    if (d.fit_b[t][d.n_fit]) im.fit_bout[t] = (float)d.fit_b[t][d.n_fit][0];
  }
  DPGB_TRY(im.fit_w16.alloc(sizeof(__nv_bfloat16) * w16.size()));
  DPGB_TRY(im.fit_f32.alloc(sizeof(float) * f32.size()));
  DPGB_CUDA(cudaMemcpy(im.fit_w16.ptr, w16.data(), sizeof(__nv_bfloat16) * w16.size(), cudaMemcpyHostToDevice));
  DPGB_CUDA(cudaMemcpy(im.fit_f32.ptr, f32.data(), sizeof(float) * f32.size(), cudaMemcpyHostToDevice));
  const __nv_bfloat16* w = im.fit_w16.as<__nv_bfloat16>();
  const float* f = im.fit_f32.as<float>();
  for (int l = 0; l < d.n_fit; ++l) {
    im.fit_Wt[l] = w + offWt[l];
    im.fit_Wb[l] = w + offWb[l];
    im.fit_b[l] = f + offb[l];
    im.fit_idt[l] = offi[l] == (size_t)-1 ? nullptr : f + offi[l];
  }
  im.fit_wout = f + offw;
  im.use_fit_tc = 1;
  return DPGB_OK;
}

// forward + input-gradient backward of the fitting of all typed rows on the
// tensor cores, one launch per layer (each 128-row tile uses its type's
// weights).  Db: BF16 descriptors (sorted rows); dD: FP32 output.
// With dxyz set (axis width 16), the last backward GEMM is folded into
// dE/dxyz (launch_fit_dxyz) and dD is not written; *dxyz_done says so.
int run_fit_tc(DeepPotImpl& dp, int nrows, const __nv_bfloat16* Db, float* dD, float* act, float* gbuf,
               __nv_bfloat16* fitb, double* e_sorted, int* err, cudaStream_t st, float* dxyz, const float* xyz,
               int* dxyz_done) {
  const int nh = dp.fit_nh, dim = dp.fit_width[0], nt = dp.desc.ntypes;
  int maxw = 0;
  for (int l = 1; l <= nh; ++l) maxw = std::max(maxw, dp.fit_width[l]);
  const size_t plane = (size_t)nrows * maxw;
  auto Yf = [&](int l) { return act + (size_t)l * plane; };
  auto Tt = [&](int l) { return act + (size_t)(nh + l) * plane; };
  // BF16 planes (fit_bf16_planes of them): the hidden outputs' high and low
  // parts, two ping-pong gradient planes and the low part of the gradient
  // the first layer's backward reads
  auto Yb = [&](int l) { return fitb + (size_t)l * plane; };
  auto Yb_lo = [&](int l) { return fitb + (size_t)(nh + l) * plane; };
  auto dPb = [&](int k) { return fitb + (size_t)(2 * nh + k) * plane; };
  __nv_bfloat16* dP1_lo = fitb + (size_t)(2 * nh + 2) * plane;
  auto dX = [&](int k) { return gbuf + (size_t)k * plane; };
  FitGemm base{};
  base.ntypes = nt;
  base.tile0[0] = 0;
  for (int t = 0; t < nt; ++t) {
    base.row0[t] = dp.type_off[t];
    base.tile0[t + 1] = base.tile0[t] + ceil_div(dp.type_count[t], 128);
    base.b_out[t] = dp.fit_bout[t];
  }
  base.row0[nt] = dp.type_off[nt];
  for (int l = 0; l < nh; ++l) {
    const int a = dp.fit_width[l], o = dp.fit_width[l + 1];
    FitGemm g = base;
    g.mode = l == nh - 1 ? kFitFwdLast : kFitFwd;
    g.N = o;
    g.K = a;
    g.Kp = pad64(a);
    g.A = l == 0 ? Db : Yb(l - 1);
    g.lda = l == 0 ? dim : maxw;
    // D (BF16, its rounding is harmless) . (W hi + W lo); the hidden outputs
    // in split BF16 as well
    if (l > 0) g.A_lo = Yb_lo(l - 1);
    if (l < nh - 1) g.Yb_lo = Yb_lo(l);
    g.B = dp.fit_Wt[l];
    g.bias = dp.fit_b[l];
    g.idt = dp.fit_idt[l];
    g.skip = (o == a && l > 0) ? 1 : 0;
    g.Xs = l > 0 ? Yf(l - 1) : nullptr;
    g.ldxs = maxw;
    g.Yf = Yf(l);
    g.Yb = Yb(l);
    g.Tt = Tt(l);
    g.ldy = maxw;
    if (g.mode == kFitFwdLast) {
      g.w_out = dp.fit_wout;
      g.e_out = e_sorted;
      g.dPb = dPb(0);
      if (nh == 1) g.dPb_lo = dP1_lo;  // read by the first layer's backward
    }
    DPGB_TRY(launch_fit_gemm(g, err, st));
  }
  // backward through the hidden layers nh-1 .. 1 (dP ping-pongs between two planes)
  int cur = 0;
  for (int l = nh - 1; l >= 1; --l) {
    const int a = dp.fit_width[l], o = dp.fit_width[l + 1];
    FitGemm g = base;
    g.mode = kFitBwd;
    g.N = a;
    g.K = o;
    g.Kp = pad64(o);
    // dP (BF16) . (W hi + W lo)
    g.A = dPb(cur);
    g.lda = maxw;
    g.B = dp.fit_Wb[l];
    if (l == 1) g.dPb_lo = dP1_lo;  // the gradient the first layer's backward reads
    if (o == a) {  // skip connection of layer l: gradient of its output passes through
      if (l == nh - 1) {
        g.dYup = dp.fit_wout;  // [type][wl] broadcast over rows
        g.lddyup = 0;
      } else {
        g.dYup = dX((cur + 1) & 1);
        g.lddyup = maxw;
      }
    }
    const bool lower_skip = dp.fit_width[l] == dp.fit_width[l - 1];
    g.dXf = lower_skip ? dX(cur) : nullptr;
    g.T_lo = Tt(l - 1);
    g.idt_lo = dp.fit_idt[l - 1];
    g.ldy = maxw;
    g.dPb = dPb(cur ^ 1);
    DPGB_TRY(launch_fit_gemm(g, err, st));
    cur ^= 1;
  }
  *dxyz_done = 0;
  if (dxyz && dp.desc.axis_neuron == 16 && dim == 16 * dp.ng && dp.fit_width[1] <= 256) {
    FitDxyz f{};
    f.ntypes = base.ntypes;
    for (int t = 0; t <= base.ntypes; ++t) {
      f.row0[t] = base.row0[t];
      f.tile0[t] = base.tile0[t];
    }
    f.K = dp.fit_width[1];
    f.Kp = pad64(f.K);
    f.ng = dp.ng;
    f.nnei = dp.sel.nnei;
    f.A = dPb(cur);
    f.A_lo = dP1_lo;
    f.lda = maxw;
    f.B = dp.fit_Wb[0];
    f.xyz = xyz;
    f.sorted_rows = dp.sorted_rows_dev.as<int>();
    f.dxyz = dxyz;
    DPGB_TRY(launch_fit_dxyz(f, err, st));
    *dxyz_done = 1;
    return DPGB_OK;
  }
  FitGemm g = base;
  g.mode = kFitStore;
  g.N = dim;
  g.K = dp.fit_width[1];
  g.Kp = pad64(g.K);
  g.A = dPb(cur);
  g.A_lo = dP1_lo;
  g.lda = maxw;
  g.B = dp.fit_Wb[0];
  g.out = dD;
  g.ldo = dim;
  return launch_fit_gemm(g, err, st);
}

int validate_desc(const dpgb_se_a_desc* d) {
  if (!d) return fail(DPGB_EINVAL, "NULL model description");
  if (d->ntypes <= 0 || d->ntypes > DPGB_MAX_TYPES) return fail(DPGB_EINVAL, "ntypes out of range");
  if (d->n_emb <= 0 || d->n_emb > kMaxEmbLayers) return fail(DPGB_EINVAL, "1..4 embedding layers are supported");
  for (int l = 0; l < d->n_emb; ++l)
    if (d->emb_neuron[l] <= 0 || d->emb_neuron[l] > 128)
      return fail(DPGB_EINVAL, "embedding widths must be in 1..128");
  if (d->n_fit <= 0 || d->n_fit > kMaxFitLayers) return fail(DPGB_EINVAL, "1..5 hidden fitting layers are supported");
  const int ng = d->emb_neuron[d->n_emb - 1];
  if (d->axis_neuron <= 0 || d->axis_neuron > ng) return fail(DPGB_EINVAL, "bad axis_neuron");
  if (d->dim_descrpt != ng * d->axis_neuron) return fail(DPGB_EINVAL, "dim_descrpt != ng * axis_neuron");
  if (!(d->rcut_smth < d->rcut)) return fail(DPGB_EINVAL, "rmin should be less than rmax.");
  if (!d->davg || !d->dstd || !d->atom_ener_bias) return fail(DPGB_EINVAL, "missing davg/dstd/bias");
  int nnei = 0;
  for (int t = 0; t < d->ntypes; ++t) nnei += d->sel[t];
  if (nnei <= 0 || nnei > 1024) return fail(DPGB_EINVAL, "sum(sel) must be in 1..1024");
  return DPGB_OK;
}

template <typename T>
int build_dev_model(DeepPotImpl& dp, DevModel<T>& m) {
  const dpgb_se_a_desc& d = dp.desc;
  const int nt = d.ntypes, nnei = dp.sel.nnei;
  const int nnets = dp.nnets;
  // embedding: W[l] [nnets, nin, nout]
  int nin = 1;
  m.emb.n_layer = d.n_emb;
  for (int l = 0; l < d.n_emb; ++l) {
    const int nout = d.emb_neuron[l];
    m.emb.width[l] = nout;
    std::vector<double> W((size_t)nnets * nin * nout), b((size_t)nnets * nout), idt;
    bool has_idt = false;
    for (int e = 0; e < nnets; ++e) has_idt |= d.emb_idt[e][l] != nullptr;
    if (has_idt) idt.assign((size_t)nnets * nout, 1.0);
    for (int e = 0; e < nnets; ++e) {
      if (!d.compressed && (!d.emb_w[e][l] || !d.emb_b[e][l])) return fail(DPGB_EINVAL, "missing embedding weights");
      if (d.emb_w[e][l]) std::copy(d.emb_w[e][l], d.emb_w[e][l] + (size_t)nin * nout, W.begin() + (size_t)e * nin * nout);
      if (d.emb_b[e][l]) std::copy(d.emb_b[e][l], d.emb_b[e][l] + nout, b.begin() + (size_t)e * nout);
      if (d.emb_idt[e][l]) std::copy(d.emb_idt[e][l], d.emb_idt[e][l] + nout, idt.begin() + (size_t)e * nout);
    }
    m.emb.W[l] = m.upload(W);
    m.emb.b[l] = m.upload(b);
    m.emb.idt[l] = has_idt ? m.upload(idt) : nullptr;
    if (!m.emb.W[l] || !m.emb.b[l]) return fail(DPGB_ENOMEM, "weight upload failed");
    nin = nout;
  }
  // compressed tables
  m.emb.compressed = d.compressed;
  if (d.compressed) {
    std::vector<double> tab;
    std::vector<TabMeta<T>> meta(nnets);
    for (int e = 0; e < nnets; ++e) {
      const double* info = d.table_info[e];
      if (!d.table[e] || !(info[3] > 0) || !(info[4] > 0)) return fail(DPGB_EINVAL, "missing compression table");
      TabMeta<T> tm;
      tm.lower = (T)info[0];
      tm.upper = (T)info[1];
      tm.mx = (T)info[2];
      tm.s0 = (T)info[3];
      tm.s1 = (T)info[4];
      tm.first = (int)((tm.upper - tm.lower) / tm.s0);
      const T bxx = std::nextafter(tm.mx, tm.lower);
      tm.hi_idx = tm.first + (int)((bxx - tm.upper) / tm.s1);
      tm.hi_xx = tm.mx - ((tm.hi_idx - tm.first) * tm.s1 + tm.upper);
      tm.offset = (long long)tab.size();
      const long long nspline = (long long)tm.hi_idx + 1;
      tab.insert(tab.end(), d.table[e], d.table[e] + nspline * 6 * dp.ng);
      meta[e] = tm;
    }
    m.emb.table = m.upload(tab);
    auto* b = new DeviceBuffer();
    m.owned.push_back(b);
    DPGB_TRY(b->alloc(sizeof(TabMeta<T>) * nnets));
    DPGB_CUDA(cudaMemcpy(b->ptr, meta.data(), sizeof(TabMeta<T>) * nnets, cudaMemcpyHostToDevice));
    m.emb.meta = b->as<TabMeta<T>>();
  }
  // fitting: W[l] [nt, nin, nout]
  m.fit.n_hidden = d.n_fit;
  m.fit.width[0] = d.dim_descrpt;
  for (int l = 0; l < d.n_fit; ++l) m.fit.width[l + 1] = d.fit_neuron[l];
  for (int l = 0; l < d.n_fit; ++l) {
    const int a = m.fit.width[l], o = m.fit.width[l + 1];
    std::vector<double> W((size_t)nt * a * o), b((size_t)nt * o), idt;
    bool has_idt = false;
    for (int t = 0; t < nt; ++t) has_idt |= d.fit_idt[t][l] != nullptr;
    if (has_idt) idt.assign((size_t)nt * o, 1.0);
    for (int t = 0; t < nt; ++t) {
      if (!d.fit_w[t][l] || !d.fit_b[t][l]) return fail(DPGB_EINVAL, "missing fitting weights");
      std::copy(d.fit_w[t][l], d.fit_w[t][l] + (size_t)a * o, W.begin() + (size_t)t * a * o);
      std::copy(d.fit_b[t][l], d.fit_b[t][l] + o, b.begin() + (size_t)t * o);
      if (d.fit_idt[t][l]) std::copy(d.fit_idt[t][l], d.fit_idt[t][l] + o, idt.begin() + (size_t)t * o);
    }
    m.fit.W[l] = m.upload(W);
    m.fit.b[l] = m.upload(b);
    m.fit.idt[l] = has_idt ? m.upload(idt) : nullptr;
  }
  {
    const int wl = m.fit.width[d.n_fit];
    std::vector<double> w((size_t)nt * wl), b(nt, 0.0);
    for (int t = 0; t < nt; ++t) {
      if (!d.fit_w[t][d.n_fit]) return fail(DPGB_EINVAL, "missing output layer");
      std::copy(d.fit_w[t][d.n_fit], d.fit_w[t][d.n_fit] + wl, w.begin() + (size_t)t * wl);
      if (d.fit_b[t][d.n_fit]) b[t] = d.fit_b[t][d.n_fit][0];
    }
    m.fit.w_out = m.upload(w);
    m.fit.b_out = m.upload(b);
  }
  std::vector<double> avg(d.davg, d.davg + (size_t)nt * nnei * 4), sd(d.dstd, d.dstd + (size_t)nt * nnei * 4);
  m.davg = m.upload(avg);
  m.dstd = m.upload(sd);
  std::vector<double> isd(sd.size());
  for (size_t k = 0; k < sd.size(); ++k) isd[k] = 1.0 / sd[k];
  m.dstd_inv = m.upload(isd);
  return DPGB_OK;
}

// stable sort of the integer image shifts by norm (ties keep enumeration order)
std::vector<int> default_shifts(const int nbuff[3]) {
  std::vector<int> xyz;
  for (int x = -nbuff[0]; x <= nbuff[0]; ++x)
    for (int y = -nbuff[1]; y <= nbuff[1]; ++y)
      for (int z = -nbuff[2]; z <= nbuff[2]; ++z) {
        xyz.push_back(x);
        xyz.push_back(y);
        xyz.push_back(z);
      }
  const int n = (int)xyz.size() / 3;
  std::vector<int> idx(n);
  std::iota(idx.begin(), idx.end(), 0);
  std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) {
    const double na = std::sqrt((double)(xyz[3 * a] * xyz[3 * a] + xyz[3 * a + 1] * xyz[3 * a + 1] + xyz[3 * a + 2] * xyz[3 * a + 2]));
    const double nb = std::sqrt((double)(xyz[3 * b] * xyz[3 * b] + xyz[3 * b + 1] * xyz[3 * b + 1] + xyz[3 * b + 2] * xyz[3 * b + 2]));
    return na < nb;
  });
  std::vector<int> out;
  for (int i : idx) {
    out.push_back(xyz[3 * i]);
    out.push_back(xyz[3 * i + 1]);
    out.push_back(xyz[3 * i + 2]);
  }
  return out;
}

// Size buckets of a batch's frames (atoms <= 128, <= 512, <= 2048, more)
// and the work-item size chosen for each: a bucket's rows (of each centre
// type) are cut into items of at most tile_rows rows; 0 leaves them to the
// default split (about 3 x SMs near-equal items over all rows)
struct BatchPlan {
  std::vector<int> row_bucket;  // bucket of every batch row
  int tile_rows[DPGB_BATCH_BUCKETS] = {0, 0, 0, 0};
  unsigned long long version = 0;  // from plan_versions: unique over the process
  bool tiled() const {
    for (int k = 0; k < DPGB_BATCH_BUCKETS; ++k)
      if (tile_rows[k] > 0) return true;
    return false;
  }
};

std::atomic<unsigned long long> plan_versions{0};

int bucket_of(int natoms) {
  return natoms <= 128 ? 0 : natoms <= 512 ? 1 : natoms <= 2048 ? 2 : 3;
}

// plan: a batch's buckets and tiles (NULL: one system, or a batch without
// tiles).  The rows of each type are ordered by bucket, then row, and the
// work items of a tiled plan are taken from a queue, largest first.
int prepare_types(DeepPotImpl& dp, int nframes, int natom, const int* atype_host, cudaStream_t st,
                  const BatchPlan* plan = nullptr) {
  if (plan && !plan->tiled()) plan = nullptr;
  const bool same = dp.cached_nframes == nframes && (int)dp.atype_cache.size() == natom &&
                    std::equal(dp.atype_cache.begin(), dp.atype_cache.end(), atype_host) &&
                    dp.plan_owner == plan && (!plan || dp.plan_version == plan->version);
  if (same) return DPGB_OK;
  if (plan && (nframes != 1 || (int)plan->row_bucket.size() != natom))
    return fail(DPGB_EINVAL, "batch plan does not match the rows");
  ++dp.gen;
  dp.cached_nframes = -1;  // until the preparation below completes
  dp.plan_owner = plan;
  dp.plan_version = plan ? plan->version : 0;
  const int nt = dp.desc.ntypes;
  for (int i = 0; i < natom; ++i)
    if (atype_host[i] >= nt) return fail(DPGB_EINVAL, "atom type out of range");
  dp.atype_cache.assign(atype_host, atype_host + natom);
  dp.type_count.assign(nt, 0);
  for (int i = 0; i < natom; ++i)
    if (atype_host[i] >= 0) dp.type_count[atype_host[i]] += nframes;
  dp.type_off.assign(nt + 1, 0);
  for (int t = 0; t < nt; ++t) dp.type_off[t + 1] = dp.type_off[t] + dp.type_count[t];
  // sorted position of every (frame, atom): by type, then frame, then atom
  dp.row_pos_h.assign((size_t)nframes * natom, 0);
  std::vector<int> cur(dp.type_off.begin(), dp.type_off.end() - 1);
  if (plan) {
    for (int t = 0; t < nt; ++t)
      for (int k = 0; k < DPGB_BATCH_BUCKETS; ++k)
        for (int i = 0; i < natom; ++i)
          if (atype_host[i] == t && plan->row_bucket[i] == k) dp.row_pos_h[i] = cur[t]++;
  } else {
    for (int t = 0; t < nt; ++t)
      for (int f = 0; f < nframes; ++f)
        for (int i = 0; i < natom; ++i)
          if (atype_host[i] == t) dp.row_pos_h[(size_t)f * natom + i] = cur[t]++;
  }
  // inverse map (sorted position -> row) of the typed rows
  const int nsorted = dp.type_off[nt];
  std::vector<int> sorted_rows((size_t)std::max(nsorted, 1), 0);
  for (int f = 0; f < nframes; ++f)
    for (int i = 0; i < natom; ++i)
      if (atype_host[i] >= 0) sorted_rows[dp.row_pos_h[(size_t)f * natom + i]] = f * natom + i;
  // work chunks of the tensor-core embedding: contiguous sorted rows of one
  // centre type.  The embedding kernels run one CTA per chunk with three
  // CTAs per SM, so the rows are cut into at most 3 x SMs chunks of
  // near-equal size (a CTA that had to take a second chunk would double the
  // launch).  The table kernels (compressed nets) run one persistent CTA
  // per SM that stages each section's table rows for a chunk behind a
  // barrier, where its warps wait for the slowest: they take SMs chunks,
  // one per CTA (three per CTA had cost 0.2 ms of barrier waits in the
  // 98,304-atom step).
  std::vector<WorkChunk> chunks;
  {
    int dev = 0, nsm = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int slots = std::max(1, (dp.use_tab && !plan ? 1 : 3) * nsm);
    std::vector<int> per(nt, 0);
    std::vector<double> rem(nt, 0.0);
    int used = 0;
    for (int t = 0; t < nt; ++t) {
      const int n = dp.type_off[t + 1] - dp.type_off[t];
      if (n <= 0) continue;
      const double share = nsorted > 0 ? (double)slots * n / nsorted : 0.0;
      per[t] = std::max(1, std::min(n, (int)share));
      rem[t] = share - per[t];
      used += per[t];
    }
    while (used < slots) {  // largest remainder first
      int best = -1;
      for (int t = 0; t < nt; ++t) {
        const int n = dp.type_off[t + 1] - dp.type_off[t];
        if (per[t] < n && (best < 0 || rem[t] > rem[best])) best = t;
      }
      if (best < 0) break;
      ++per[best];
      rem[best] -= 1.0;
      ++used;
    }
    auto cut = [&](int r0, int n, int pieces, int t) {
      for (int k = 0; k < pieces; ++k) {
        const int a = r0 + (int)((long long)k * n / pieces), b = r0 + (int)((long long)(k + 1) * n / pieces);
        if (b > a) chunks.push_back(WorkChunk{a, b, t, 0});
      }
    };
    if (!plan) {
      for (int t = 0; t < nt; ++t) cut(dp.type_off[t], dp.type_off[t + 1] - dp.type_off[t], per[t], t);
    } else {
      // per (type, bucket) segment of the sorted rows: items of at most the
      // bucket's tile rows, or the type's default share of items
      for (int t = 0; t < nt; ++t) {
        const int r0 = dp.type_off[t], r1 = dp.type_off[t + 1];
        for (int a = r0; a < r1;) {
          const int k = plan->row_bucket[sorted_rows[a]];
          int b = a;
          while (b < r1 && plan->row_bucket[sorted_rows[b]] == k) ++b;
          const int n = b - a, tile = plan->tile_rows[k];
          const int pieces = tile > 0 ? (n + tile - 1) / tile
                                      : std::max(1, (int)((long long)per[t] * n / std::max(r1 - r0, 1)));
          cut(a, n, pieces, t);
          a = b;
        }
      }
      // largest items first: the queue hands the small ones out at the end
      std::stable_sort(chunks.begin(), chunks.end(),
                       [](const WorkChunk& x, const WorkChunk& y) { return x.row1 - x.row0 > y.row1 - y.row0; });
    }
  }
  dp.nchunks = (int)chunks.size();
  dp.use_queue = plan ? 1 : 0;
  if (dp.use_queue) DPGB_TRY(dp.queue_dev.alloc(2 * sizeof(int)));
  DPGB_TRY(dp.row_pos_dev.alloc(sizeof(int) * dp.row_pos_h.size()));
  DPGB_TRY(dp.atype_dev.alloc(sizeof(int) * natom));
  DPGB_TRY(dp.sorted_rows_dev.alloc(sizeof(int) * sorted_rows.size()));
  DPGB_TRY(dp.chunks_dev.alloc(sizeof(WorkChunk) * std::max<size_t>(chunks.size(), 1)));
  DPGB_CUDA(cudaMemcpyAsync(dp.row_pos_dev.ptr, dp.row_pos_h.data(), sizeof(int) * dp.row_pos_h.size(),
                            cudaMemcpyHostToDevice, st));
  DPGB_CUDA(cudaMemcpyAsync(dp.atype_dev.ptr, atype_host, sizeof(int) * natom, cudaMemcpyHostToDevice, st));
  DPGB_CUDA(cudaMemcpyAsync(dp.sorted_rows_dev.ptr, sorted_rows.data(), sizeof(int) * sorted_rows.size(),
                            cudaMemcpyHostToDevice, st));
  if (!chunks.empty())
    DPGB_CUDA(cudaMemcpyAsync(dp.chunks_dev.ptr, chunks.data(), sizeof(WorkChunk) * chunks.size(),
                              cudaMemcpyHostToDevice, st));
  DPGB_CUDA(cudaStreamSynchronize(st));  // host vectors may change on the next call
  dp.cached_nframes = nframes;
  return DPGB_OK;
}

// the queue counters of the two persistent kernels (NULL without a queue)
int* queue_fwd(DeepPotImpl& dp) { return dp.use_queue ? dp.queue_dev.as<int>() : nullptr; }
int* queue_bwd(DeepPotImpl& dp) { return dp.use_queue ? dp.queue_dev.as<int>() + 1 : nullptr; }

// An external neighbour list with explicit ghost atoms (one frame): device
// coordinates / types of all nall atoms (local first) and a CSR list over
// the local atoms.
struct ExtList {
  const double* coord;
  const int* atype;
  int nall;
  const int* off;
  const int* idx;
  int sorted;
};

// A batch of periodic frames of different sizes (device tables prepared once;
// the evaluation itself only launches kernels, so it can be captured in a
// CUDA graph).  The frames' atoms are the rows of one "frame" of natoms.
struct BatchIn {
  FrameTab ft;
  int ncells;
  const double* svec;
  const int* spos;
  int max_atoms;  // atoms of the largest frame
  int nsvec;      // shift vectors of all frames
};

template <typename T>
int run(DeepPotImpl& dp, DevModel<T>& m, int nframes, int natom, const double* coord_dev, const double* box_host,
        double* energy, double* force, double* virial, double* atom_energy, double* atom_virial, cudaStream_t st,
        const ExtList* ext = nullptr, const BatchIn* batch = nullptr) {
  const dpgb_se_a_desc& d = dp.desc;
  const int nnei = dp.sel.nnei;
  const long long nrows = (long long)nframes * natom;
  if (nrows >= (1LL << 31) / std::max(nnei, 1)) return fail(DPGB_EINVAL, "too many atoms for 32-bit pair ids");
  if ((ext || batch) && nframes != 1) return fail(DPGB_EINVAL, "an external list or a batch runs as one frame");
  ++dp.evals;
  int launches = 0;
  const bool own_geom = !ext && !batch;
  const bool skin_on = own_geom && box_host && dp.skin > 0.0;
  const double rc_geo = skin_on ? d.rcut + dp.skin : d.rcut;  // list radius of the cell search
  // --- geometry (host) ---
  std::vector<CellGeom> geo(own_geom ? nframes : 0);
  std::vector<std::vector<int>> spos(own_geom ? nframes : 0);
  int nshift_max = 1;
  std::vector<std::vector<double>> svecs(nframes);
  std::vector<double> host_coord;
  if (own_geom && box_host) DPGB_TRY(check_finite(box_host, 9 * (size_t)nframes, "cell"));
  for (int f = 0; f < (int)geo.size(); ++f) {
    if (box_host) {
      CellGeom g0;
      DPGB_TRY(box_geom(box_host + 9 * f, g0));
      // reference image range from the face distances
      CellGeom tmp;
      std::vector<int> dummy;
      double face_rc = rc_geo;
      // nbuff = ceil(rcut / face distance)
      const double* c = box_host + 9 * f;
      auto crn = [&](int p, int q) {
        const double x = c[p * 3 + 1] * c[q * 3 + 2] - c[p * 3 + 2] * c[q * 3 + 1];
        const double y = c[p * 3 + 2] * c[q * 3 + 0] - c[p * 3 + 0] * c[q * 3 + 2];
        const double z = c[p * 3 + 0] * c[q * 3 + 1] - c[p * 3 + 1] * c[q * 3 + 0];
        return std::sqrt(x * x + y * y + z * z);
      };
      const double vol = std::fabs(c[0] * (c[4] * c[8] - c[5] * c[7]) - c[1] * (c[3] * c[8] - c[5] * c[6]) +
                                   c[2] * (c[3] * c[7] - c[4] * c[6]));
      const int nb[3] = {(int)std::ceil(face_rc / (vol / crn(1, 2))), (int)std::ceil(face_rc / (vol / crn(2, 0))),
                         (int)std::ceil(face_rc / (vol / crn(0, 1)))};
      const std::vector<int> shifts = default_shifts(nb);
      const int ns = (int)shifts.size() / 3;
      DPGB_TRY(periodic_geom(box_host + 9 * f, rc_geo, ns, shifts.data(), geo[f], spos[f]));
      shift_vectors(geo[f], shifts.data(), ns, svecs[f]);
      nshift_max = std::max(nshift_max, ns);
      (void)tmp;
      (void)dummy;
    } else {
      if (host_coord.empty()) {
        host_coord.resize((size_t)nframes * natom * 3);
        DPGB_CUDA(cudaMemcpyAsync(host_coord.data(), coord_dev, sizeof(double) * host_coord.size(),
                                  cudaMemcpyDeviceToHost, st));
        DPGB_CUDA(cudaStreamSynchronize(st));
      }
      DPGB_TRY(check_finite(host_coord.data() + (size_t)f * natom * 3, (size_t)natom * 3, "coordinate"));
      DPGB_TRY(open_geom(host_coord.data() + (size_t)f * natom * 3, natom, d.rcut, geo[f]));
      spos[f].assign(1, 0);
      svecs[f].assign(3, 0.0);
    }
  }
  // --- device workspace ---
  size_t cell_bytes = 0;
  for (int f = 0; f < (int)geo.size(); ++f) cell_bytes = std::max(cell_bytes, nlist_pt_workspace(natom, geo[f]));
  const long long npair = nrows * nnei;
  if (npair >= (1LL << 31)) return fail(DPGB_EINVAL, "more than 2^31 neighbour slots in one evaluation");
  // transpose keys: local rows (ghost images fold onto their atom), or every
  // explicit extended atom with an external list (forces on ghosts returned)
  const long long nkeys = ext ? (long long)ext->nall : nrows;
  const int ng = dp.ng, dim = dp.dim;
  int maxw = 0;
  for (int l = 1; l <= m.fit.n_hidden; ++l) maxw = std::max(maxw, m.fit.width[l]);
  if (batch) cell_bytes = nlist_batch_workspace(natom, batch->ncells);
  DPGB_TRY(dp.ws_cell.alloc(cell_bytes));
  DPGB_TRY(dp.ws_nlist.alloc(sizeof(int) * npair));
  // the mixed form's model-list forces without atomic virials go through
  // the fixed-point scatter; every other gather reads the sorted transpose
  // (a batch: when the tensor-core or table backward adds the gradients
  // itself, which finds each row's frame)
  const bool fused_bwd = std::is_same<T, float>::value && (dp.use_tc != 0 || dp.use_tab != 0);
  // (an external list: every explicit extended atom gets its force, as the
  // transpose path gives it)
  const bool scatter =
      std::is_same<T, float>::value && !atom_virial && (own_geom || ((batch || ext) && fused_bwd));
  if (scatter) {
    DPGB_TRY(dp.ws_facc.alloc(sizeof(unsigned long long) * 3 * nkeys));
  } else {
    DPGB_TRY(dp.ws_keys.alloc(sizeof(int) * npair));
    DPGB_TRY(dp.ws_tr.alloc(transpose_workspace(npair, (int)nkeys)));
  }
  DPGB_TRY(dp.ws_status.alloc(sizeof(int) * kStatusSlots));
  DPGB_TRY(dp.ws_coord.alloc(sizeof(double) * nrows * 3));
  DPGB_TRY(dp.ws_svec.alloc(sizeof(double) * 3 * (size_t)nshift_max * nframes));
  size_t spos_n = 0;
  for (auto& v : spos) spos_n = std::max(spos_n, v.size());
  DPGB_TRY(dp.ws_spos.alloc(sizeof(int) * spos_n * nframes));
  DPGB_TRY(dp.ws_D.alloc(sizeof(T) * nrows * dim));
  DPGB_TRY(dp.ws_dD.alloc(sizeof(T) * nrows * dim));
  DPGB_TRY(dp.ws_xyz.alloc(sizeof(T) * nrows * 4 * ng));
  DPGB_TRY(dp.ws_g.alloc(sizeof(T) * npair * 3));
  DPGB_TRY(dp.ws_vir.alloc(sizeof(double) * nrows * 9));
  DPGB_TRY(dp.ws_erow.alloc(sizeof(double) * nrows));
  DPGB_TRY(dp.ws_esorted.alloc(sizeof(double) * nrows));
  const int sum_frames = batch ? batch->ft.nframes : nframes;
  const int sum_chunk = frame_chunk((long long)sum_frames * (batch ? batch->max_atoms : natom), batch != nullptr);
  const int sum_chunks = ceil_div(batch ? batch->max_atoms : natom, sum_chunk);
  DPGB_TRY(dp.ws_part.alloc(sizeof(double) * 10 * (size_t)sum_frames * sum_chunks));
  DPGB_TRY(dp.ws_act.alloc(sizeof(T) * 2 * m.fit.n_hidden * nrows * maxw));
  DPGB_TRY(dp.ws_gbuf.alloc(sizeof(T) * 4 * nrows * maxw));
  // skin-list state: candidate capacities, buffers, and whether the stored
  // candidates still belong to this system (else the next evaluation builds)
  int ncand = 0;
  double skin_margin = 0.0;
  if (skin_on) {
    if (dp.skin_grow > 0) {  // a row needed skin_grow slots: widen past that
      dp.skin_factor *= std::max(1.5, 1.1 * dp.skin_grow / std::max(dp.skin_sel.nnei, 1));
      dp.skin_grow = 0;
      dp.skin_nframes = -1;
    }
    // flat candidate rows: sum(sel) scaled by the volume ratio of the two
    // spheres and skin_factor
    const double growth = std::pow(rc_geo / d.rcut, 3) * dp.skin_factor;
    SelInfo cs = dp.sel;
    cs.nnei = (int)std::ceil(dp.sel.nnei * growth / 8.0) * 8;
    cs.strict = 1;
    cs.flat = 1;
    ncand = cs.nnei;
    if (nrows >= (1LL << 31) / std::max(ncand, 1)) return fail(DPGB_EINVAL, "too many atoms for 32-bit candidate ids");
    DPGB_TRY(dp.ws_gate.alloc(sizeof(int) * 2));
    DPGB_TRY(dp.ws_cand.alloc(sizeof(int) * nrows * ncand));
    DPGB_TRY(dp.ws_skin_off.alloc(sizeof(double) * nrows * 3));
    DPGB_TRY(dp.ws_skin_ref.alloc(sizeof(double) * nrows * 3));
    DPGB_TRY(dp.ws_coordf.alloc(sizeof(float4) * nrows));
    DPGB_TRY(dp.ws_coordflo.alloc(sizeof(float4) * nrows));
    DPGB_TRY(dp.ws_svecf.alloc(sizeof(float4) * (size_t)nshift_max * nframes));
    DPGB_TRY(dp.ws_svecflo.alloc(sizeof(float4) * (size_t)nshift_max * nframes));
    const std::vector<double> box_now(box_host, box_host + 9 * (size_t)nframes);
    const void* ptrs = dp.ws_cand.ptr;
    const bool same = dp.skin_nframes == nframes && dp.skin_box == box_now && dp.skin_atype == dp.atype_cache &&
                      dp.skin_cand_ptr == ptrs && dp.skin_sel.nnei == cs.nnei;
    if (!same) {
      const int init[2] = {0, -1};  // no rebuild flagged yet, no list
      DPGB_CUDA(cudaMemcpyAsync(dp.ws_gate.ptr, init, sizeof(init), cudaMemcpyHostToDevice, st));
      dp.skin_nframes = nframes;
      dp.skin_box = box_now;
      dp.skin_atype = dp.atype_cache;
      dp.skin_cand_ptr = ptrs;
      dp.skin_sel = cs;
    }
    // FP32 prefilter margin above rcut: the FP32 rounding of coordinates and
    // shift vectors of magnitude <= cmax stays below 4e-7 cmax in a distance
    double cmax = 0.0;
    for (int f = 0; f < nframes; ++f) {
      const double* c = box_host + 9 * f;
      double len = 0.0;
      for (int k = 0; k < 3; ++k) len += std::sqrt(c[3 * k] * c[3 * k] + c[3 * k + 1] * c[3 * k + 1] + c[3 * k + 2] * c[3 * k + 2]);
      const int nbm = std::max(geo[f].nbuff[0], std::max(geo[f].nbuff[1], geo[f].nbuff[2]));
      cmax = std::max(cmax, len * (nbm + 2) + dp.skin);
    }
    skin_margin = 1e-3 + 1e-6 * cmax;
  }

  int* status = dp.ws_status.as<int>();
  DPGB_CUDA(cudaMemsetAsync(status, 0, sizeof(int) * kStatusSlots, st));
  // shift tables (a batch brings its own; nothing host-side may run inside
  // a captured batch evaluation)
  if (own_geom && !dp.capturing) {  // a capture replays the tables its plain run uploaded
    std::vector<double> sv((size_t)3 * nshift_max * nframes, 0.0);
    std::vector<int> sp(spos_n * nframes, -1);
    for (int f = 0; f < (int)spos.size(); ++f) {
      std::copy(svecs[f].begin(), svecs[f].end(), sv.begin() + (size_t)3 * nshift_max * f);
      std::copy(spos[f].begin(), spos[f].end(), sp.begin() + spos_n * f);
    }
    DPGB_CUDA(cudaMemcpyAsync(dp.ws_svec.ptr, sv.data(), sizeof(double) * sv.size(), cudaMemcpyHostToDevice, st));
    DPGB_CUDA(cudaMemcpyAsync(dp.ws_spos.ptr, sp.data(), sizeof(int) * sp.size(), cudaMemcpyHostToDevice, st));
    if (skin_on) {  // the shifts' FP32 high and low parts
      std::vector<float4> svf((size_t)2 * nshift_max * nframes);
      const size_t nsv = (size_t)nshift_max * nframes;
      for (size_t q = 0; q < nsv; ++q) {
        const float h[3] = {(float)sv[3 * q], (float)sv[3 * q + 1], (float)sv[3 * q + 2]};
        svf[q] = make_float4(h[0], h[1], h[2], 0.f);
        svf[nsv + q] = make_float4((float)(sv[3 * q] - (double)h[0]), (float)(sv[3 * q + 1] - (double)h[1]),
                                   (float)(sv[3 * q + 2] - (double)h[2]), 0.f);
      }
      DPGB_CUDA(cudaMemcpyAsync(dp.ws_svecf.ptr, svf.data(), sizeof(float4) * nsv, cudaMemcpyHostToDevice, st));
      DPGB_CUDA(cudaMemcpyAsync(dp.ws_svecflo.ptr, svf.data() + nsv, sizeof(float4) * nsv, cudaMemcpyHostToDevice,
                                st));
    }
  }
  double* coord_n = dp.ws_coord.as<double>();
  int* nlist = dp.ws_nlist.as<int>();
  dp.mark(DPGB_STAGE_NLIST, 0, st);
  if (ext) {
    DPGB_TRY(launch_format_ext(nlist, ext->coord, ext->atype, ext->off, ext->idx, natom, ext->nall, d.rcut, dp.sel,
                               ext->sorted, status, st));
    ++launches;
  }
  if (batch) {
    DPGB_TRY(launch_nlist_batch(nlist, coord_n, coord_dev, dp.atype_dev.as<int>(), natom, batch->ncells, batch->ft,
                                batch->svec, batch->spos, d.rcut, dp.sel, dp.ws_cell.ptr, status, st));
    launches += 4;
  }
  int* gate = dp.ws_gate.as<int>();
  if (skin_on) {
    DPGB_TRY(launch_skin_check(gate, coord_dev, dp.ws_skin_ref.as<double>(), (int)nrows, dp.skin, dp.skin_every, st));
    ++launches;
  }
  for (int f = 0; f < (int)geo.size(); ++f) {
    const double* cin = coord_dev + (size_t)f * natom * 3;
    double* cout = coord_n + (size_t)f * natom * 3;
    if (skin_on) {
      // build (when gate[0]): wrap, candidates within rcut + skin; always:
      // select the list at rcut from the candidates
      const size_t a0 = (size_t)f * natom;
      const double* svf = dp.ws_svec.as<double>() + (size_t)3 * nshift_max * f;
      int* cand = dp.ws_cand.as<int>() + a0 * ncand;
      DPGB_TRY(launch_skin_coords(cout, dp.ws_coordf.as<float4>() + a0, dp.ws_coordflo.as<float4>() + a0,
                                  dp.ws_skin_off.as<double>() + 3 * a0, dp.ws_skin_ref.as<double>() + 3 * a0, cin,
                                  natom, geo[f], gate, st, status));
      DPGB_TRY(launch_nlist_pt(cand, cout, dp.atype_dev.as<int>(), natom, geo[f], dp.ws_spos.as<int>() + spos_n * f,
                               svf, rc_geo, dp.skin_sel, dp.ws_cell.ptr, status, st, gate));
      DPGB_TRY(launch_skin_select(nlist + a0 * nnei, cand, ncand, cout, dp.ws_coordf.as<float4>() + a0,
                                  dp.ws_coordflo.as<float4>() + a0, dp.atype_dev.as<int>(), svf,
                                  dp.ws_svecf.as<float4>() + (size_t)nshift_max * f,
                                  dp.ws_svecflo.as<float4>() + (size_t)nshift_max * f, natom, d.rcut, skin_margin,
                                  dp.sel, status, st));
      launches += 7;
      continue;
    }
    if (box_host) {
      DPGB_TRY(launch_normalize(cout, cin, natom, geo[f], st, status));
    } else {
      DPGB_CUDA(cudaMemcpyAsync(cout, cin, sizeof(double) * natom * 3, cudaMemcpyDeviceToDevice, st));
    }
    ++launches;
    DPGB_TRY(launch_nlist_pt(nlist + (size_t)f * natom * nnei, cout, dp.atype_dev.as<int>(), natom, geo[f],
                             dp.ws_spos.as<int>() + spos_n * f, dp.ws_svec.as<double>() + (size_t)3 * nshift_max * f,
                             d.rcut, dp.sel, dp.ws_cell.ptr, status, st));
    launches += 5;  // cell count, scan, fill, staged search, per-atom search of flagged cells
  }
  if (skin_on) {
    DPGB_TRY(launch_skin_advance(gate, st));
    ++launches;
  }
  dp.nl_nframes = own_geom ? nframes : 0;
  dp.nl_natom = natom;
  dp.nl_nshift = nshift_max;
  dp.mark(DPGB_STAGE_NLIST, 1, st);
  // sorted transpose of the list over local rows
  // the sorted transpose on the side stream: only the force gather needs it
  cudaStream_t ts = st;
  const bool fork = dp.side && !scatter;
  if (fork) {
    DPGB_CUDA(cudaEventRecord(dp.ev_fork, st));
    DPGB_CUDA(cudaStreamWaitEvent(dp.side, dp.ev_fork, 0));
    ts = dp.side;
  }
  dp.mark(DPGB_STAGE_TRANSPOSE, 0, ts);
  Transpose tr{};
  if (scatter) {
    DPGB_CUDA(cudaMemsetAsync(dp.ws_facc.ptr, 0, sizeof(unsigned long long) * 3 * nkeys, ts));
  } else if (npair > 0) {
    // image-major indices fold onto their atom; explicit extended indices
    // are their own keys
    if (batch)
      batch_keys_kernel<<<ceil_div(npair, 256), 256, 0, ts>>>(dp.ws_keys.as<int>(), nlist, npair, nnei, batch->ft);
    else
      model_keys_kernel<<<ceil_div(npair, 256), 256, 0, ts>>>(dp.ws_keys.as<int>(), nlist, (int)npair, FastDiv(nnei),
                                                               ext ? ext->nall : natom, FastDiv(ext ? ext->nall : natom));
    DPGB_TRY(check_launch("model_keys"));
    ++launches;
  }
  if (!scatter) {
    DPGB_TRY(launch_transpose(tr, dp.ws_keys.as<int>(), npair, (int)nkeys, 0, dp.ws_tr.ptr, status, ts));
    launches += 4;
  }
  dp.mark(DPGB_STAGE_TRANSPOSE, 1, ts);
  if (fork) DPGB_CUDA(cudaEventRecord(dp.ev_join, dp.side));
  // descriptor forward
  DescParams<T> p{};
  p.nloc = natom;
  p.nrows = (int)nrows;
  p.nnei = nnei;
  p.ntypes = d.ntypes;
  for (int t = 0; t <= d.ntypes; ++t) p.sec[t] = dp.sel.sec[t];
  p.type_one_side = d.type_one_side;
  p.ng = ng;
  p.axis = d.axis_neuron;
  p.pad_zero = dp.pad_zero;
  p.rcut = d.rcut;
  p.rcut_smth = d.rcut_smth;
  p.davg = m.davg;
  p.dstd = m.dstd;
  p.dstd_inv = m.dstd_inv;
  p.nloc_div = FastDiv(natom);
  p.facc = scatter ? dp.ws_facc.as<unsigned long long>() : nullptr;
  p.pair_mask = d.pair_mask ? dp.pair_mask_dev.as<int>() : nullptr;
  p.coord = coord_n;
  p.atype = dp.atype_dev.as<int>();
  p.nlist = nlist;
  p.svec = dp.ws_svec.as<double>();
  p.nshift = nshift_max;
  p.row_pos = dp.row_pos_dev.as<int>();
  if (ext) {
    p.coord_ext = ext->coord;
    p.atype_ext = ext->atype;
    p.nall = ext->nall;
  }
  if (batch) {
    p.svec = batch->svec;
    p.frame_atom_off = batch->ft.atom_off;
    p.frame_svec_off = batch->ft.svec_off;
    p.nframes_batch = batch->ft.nframes;
  }
  if constexpr (std::is_same<T, float>::value) {
    // FP32 splits of the coordinates and shifts: the mixed form's
    // displacements are taken without FP64 instructions
    const int npts = ext ? ext->nall : (int)nrows;
    const int nsv = ext ? 0 : (batch ? batch->nsvec : nshift_max * nframes);
    const double* pts = ext ? ext->coord : coord_n;
    const double* svs = batch ? batch->svec : dp.ws_svec.as<double>();
    DPGB_TRY(dp.ws_xhi.alloc(sizeof(float4) * npts));
    DPGB_TRY(dp.ws_xlo.alloc(sizeof(float4) * npts));
    DPGB_TRY(dp.ws_shi.alloc(sizeof(float4) * std::max(nsv, 1)));
    DPGB_TRY(dp.ws_slo.alloc(sizeof(float4) * std::max(nsv, 1)));
    split_points_kernel<<<ceil_div(npts, 256), 256, 0, st>>>(dp.ws_xhi.as<float4>(), dp.ws_xlo.as<float4>(), pts,
                                                             npts);
    DPGB_TRY(check_launch("split_points"));
    ++launches;
    if (nsv > 0) {
      split_points_kernel<<<ceil_div(nsv, 256), 256, 0, st>>>(dp.ws_shi.as<float4>(), dp.ws_slo.as<float4>(), svs,
                                                              nsv);
      DPGB_TRY(check_launch("split_points"));
      ++launches;
    }
    p.xhi = dp.ws_xhi.as<float4>();
    p.xlo = dp.ws_xlo.as<float4>();
    p.shi = dp.ws_shi.as<float4>();
    p.slo = dp.ws_slo.as<float4>();
  }
  // virtual rows have no sorted position: point them at row 0 only for
  // reading (the kernels never write a virtual row)
  bool tc_path = false;
  if constexpr (std::is_same<T, float>::value) tc_path = dp.use_tc != 0;
  dp.mark(DPGB_STAGE_DESC_FWD, 0, st);
  if (dp.use_queue && (tc_path || dp.use_tab)) DPGB_CUDA(cudaMemsetAsync(dp.queue_dev.ptr, 0, 2 * sizeof(int), st));
  if constexpr (std::is_same<T, float>::value) {
    if (tc_path) {
      const int nsorted = dp.type_off[d.ntypes];
      DPGB_TRY(dp.ws_runlen.alloc(sizeof(int) * (size_t)std::max(nsorted, 1) * d.ntypes));
      // one buffer serves the per-section partial xyz of the forward and,
      // after it, dE/dxyz of the backward
      DPGB_TRY(dp.ws_dxyz.alloc(sizeof(float) * nrows * 4 * ((ng + 15) / 16 * 16) * d.ntypes));
      DPGB_TRY(launch_run_lengths(dp.ws_runlen.as<int>(), nlist, dp.sorted_rows_dev.as<int>(), nsorted, nnei, dp.sel,
                                  dp.pad_zero, st));
      EmbTC e = dp.tc;
      e.d_bf16 = dp.use_fit_tc;
      DPGB_TRY(launch_emb_tc_fwd(p, e, dp.chunks_dev.as<WorkChunk>(), dp.nchunks, dp.ws_runlen.as<int>(),
                                 dp.sorted_rows_dev.as<int>(), dp.ws_xyz.as<float>(), dp.ws_dxyz.as<float>(),
                                 dp.ws_D.as<float>(), status, st, queue_fwd(dp)));
      launches += 2;
    }
  }
  bool tab_path = false;
  if constexpr (std::is_same<T, float>::value) {
    tab_path = !tc_path && dp.use_tab != 0;
    if (tab_path) {
      DPGB_TRY(dp.ws_dxyz.alloc(sizeof(float) * nrows * 4 * ng));
      DPGB_TRY(dp.ws_env.alloc(sizeof(float4) * 2 * npair));
      DPGB_TRY(launch_tab_fwd(p, m.emb, dp.chunks_dev.as<WorkChunk>(), dp.nchunks, dp.sorted_rows_dev.as<int>(),
                              dp.ws_xyz.as<float>(), dp.ws_D.ptr, dp.use_fit_tc, st, queue_fwd(dp),
                              dp.ws_env.as<float4>()));
      ++launches;
    }
  }
  if (!tc_path && !tab_path) {
    DPGB_TRY(launch_desc_fwd<T>(p, m.emb, dp.ws_D.as<T>(), dp.ws_xyz.as<T>(), desc_fwd_smem<T>(p, m.emb), st));
    ++launches;
  }
  dp.mark(DPGB_STAGE_DESC_FWD, 1, st);
  dp.mark(DPGB_STAGE_FITTING, 0, st);
  bool fit_tc = false;
  if constexpr (std::is_same<T, float>::value) fit_tc = (tc_path || tab_path) && dp.use_fit_tc;
  if (fit_tc) {
    DPGB_TRY(dp.ws_fitb.alloc(sizeof(__nv_bfloat16) * (size_t)(2 * dp.fit_nh + 3) * nrows * maxw));
  }
  int dxyz_done = 0;  // dE/dxyz already formed by the fitting's last backward GEMM
  if (fit_tc) {
    if constexpr (std::is_same<T, float>::value) {
      DPGB_TRY(dp.ws_dxyz.alloc(sizeof(float) * nrows * 4 * ng * std::max(d.ntypes, 1)));
      DPGB_TRY(run_fit_tc(dp, (int)nrows, reinterpret_cast<const __nv_bfloat16*>(dp.ws_D.ptr), dp.ws_dD.as<float>(),
                          dp.ws_act.as<float>(), dp.ws_gbuf.as<float>(), dp.ws_fitb.as<__nv_bfloat16>(),
                          dp.ws_esorted.as<double>(), status + kStatusTimeout, st,
                          (tc_path || tab_path) ? dp.ws_dxyz.as<float>() : nullptr, dp.ws_xyz.as<float>(),
                          &dxyz_done));
    }
    launches += 2 * dp.fit_nh;
  } else {
    for (int t = 0; t < d.ntypes; ++t) {
      if (dp.type_count[t] == 0) continue;
      DPGB_TRY(launch_fitting<T>(m.fit, t, dp.type_off[t], dp.type_count[t], (int)nrows, dp.ws_D.as<T>(),
                                 dp.ws_dD.as<T>(), dp.ws_act.as<T>(), dp.ws_gbuf.as<T>(), dp.ws_esorted.as<double>(),
                                 0.0, st));
      launches += 2 * m.fit.n_hidden + 2;
    }
  }
  dp.mark(DPGB_STAGE_FITTING, 1, st);
  dp.mark(DPGB_STAGE_DESC_BWD, 0, st);
  if constexpr (std::is_same<T, float>::value) {
    if (tc_path) {
      // rows of virtual atoms are never visited by the tile kernels
      DPGB_CUDA(cudaMemsetAsync(dp.ws_vir.ptr, 0, sizeof(double) * nrows * 9, st));
      if (!dxyz_done) DPGB_TRY(launch_dxyz(p, dp.ws_dD.as<float>(), dp.ws_xyz.as<float>(), dp.ws_dxyz.as<float>(), st));
      DPGB_TRY(launch_emb_tc_bwd(p, dp.tc, dp.chunks_dev.as<WorkChunk>(), dp.nchunks, dp.ws_runlen.as<int>(),
                                 dp.sorted_rows_dev.as<int>(), dp.ws_dxyz.as<float>(), dp.ws_g.as<float>(),
                                 dp.ws_vir.as<double>(), status, st, queue_bwd(dp)));
      launches += 2;
    }
    if (tab_path) {
      DPGB_CUDA(cudaMemsetAsync(dp.ws_vir.ptr, 0, sizeof(double) * nrows * 9, st));
      if (!dxyz_done) DPGB_TRY(launch_dxyz(p, dp.ws_dD.as<float>(), dp.ws_xyz.as<float>(), dp.ws_dxyz.as<float>(), st));
      DPGB_TRY(launch_tab_bwd(p, m.emb, dp.chunks_dev.as<WorkChunk>(), dp.nchunks, dp.sorted_rows_dev.as<int>(),
                              dp.ws_dxyz.as<float>(), dp.ws_g.as<float>(), dp.ws_vir.as<double>(), st,
                              queue_bwd(dp), dp.ws_env.as<float4>()));
      launches += 2;
    }
  }
  if (!tc_path && !tab_path) {
    DPGB_TRY(launch_desc_bwd<T>(p, m.emb, dp.ws_dD.as<T>(), dp.ws_xyz.as<T>(), dp.ws_g.as<T>(), dp.ws_vir.as<double>(),
                                desc_bwd_smem<T>(p, m.emb), st));
    ++launches;
  }
  dp.mark(DPGB_STAGE_DESC_BWD, 1, st);
  if (fork) DPGB_CUDA(cudaStreamWaitEvent(st, dp.ev_join, 0));  // the transpose is done
  dp.mark(DPGB_STAGE_REDUCE, 0, st);
  if (scatter) {
    if (!tab_path && !tc_path) {  // the table and tensor-core backwards added the pair gradients themselves
      force_scatter_model_kernel<<<ceil_div(nrows, kGatherWarps), kGatherWarps * 32, 0, st>>>(
          dp.ws_facc.as<unsigned long long>(), reinterpret_cast<const float*>(dp.ws_g.ptr), nlist, natom,
          FastDiv(natom), nnei, (int)nrows);
      DPGB_TRY(check_launch("force_scatter"));
      ++launches;
    }
    force_fix_kernel<<<ceil_div(3 * nkeys, 256), 256, 0, st>>>(force, dp.ws_facc.as<unsigned long long>(),
                                                                (int)(3 * nkeys));
    ++launches;
  } else if (ext) {
    if (atom_virial)
      force_gather_ext_kernel<T, true><<<ceil_div(nkeys, kGatherWarps), kGatherWarps * 32, 0, st>>>(
          force, atom_virial, dp.ws_g.as<T>(), tr, nlist, ext->coord, natom, ext->nall, nnei);
    else
      force_gather_ext_kernel<T, false><<<ceil_div(nkeys, kGatherWarps), kGatherWarps * 32, 0, st>>>(
          force, nullptr, dp.ws_g.as<T>(), tr, nlist, ext->coord, natom, ext->nall, nnei);
  } else if (batch) {
    if (atom_virial)
      force_gather_batch_kernel<T, true><<<ceil_div(nrows, kGatherWarps), kGatherWarps * 32, 0, st>>>(
          force, atom_virial, dp.ws_g.as<T>(), tr, nlist, coord_n, batch->svec, batch->ft, nnei, (int)nrows);
    else
      force_gather_batch_kernel<T, false><<<ceil_div(nrows, kGatherWarps), kGatherWarps * 32, 0, st>>>(
          force, nullptr, dp.ws_g.as<T>(), tr, nlist, coord_n, batch->svec, batch->ft, nnei, (int)nrows);
  } else {
    if (atom_virial)
      force_gather_model_kernel<T, true><<<ceil_div(nrows, kGatherWarps), kGatherWarps * 32, 0, st>>>(
          force, atom_virial, dp.ws_g.as<T>(), tr, nlist, coord_n, dp.ws_svec.as<double>(), nshift_max, natom, nnei,
          (int)nrows);
    else
      force_gather_model_kernel<T, false><<<ceil_div(nrows, kGatherWarps), kGatherWarps * 32, 0, st>>>(
          force, nullptr, dp.ws_g.as<T>(), tr, nlist, coord_n, dp.ws_svec.as<double>(), nshift_max, natom, nnei,
          (int)nrows);
  }
  DPGB_TRY(check_launch("force_gather"));
  ++launches;
  double* e_row = atom_energy ? atom_energy : dp.ws_erow.as<double>();
  atom_energy_kernel<<<ceil_div(nrows, 256), 256, 0, st>>>(e_row, dp.ws_esorted.as<double>(), dp.row_pos_dev.as<int>(),
                                                           dp.atype_dev.as<int>(), dp.bias_dev.as<double>(), natom,
                                                           (int)nrows);
  DPGB_TRY(check_launch("atom_energy"));
  frame_part_kernel<<<dim3(sum_chunks, sum_frames), kFrameSumThreads, 0, st>>>(
      dp.ws_part.as<double>(), e_row, dp.ws_vir.as<double>(), batch ? batch->ft.atom_off : nullptr, natom, sum_chunk);
  DPGB_TRY(check_launch("frame_part"));
  frame_final_kernel<<<ceil_div(sum_frames, 8), 256, 0, st>>>(energy, virial, dp.ws_part.as<double>(), sum_chunks,
                                                               sum_frames);
  DPGB_TRY(check_launch("frame_sum"));
  launches += 3;
  dp.mark(DPGB_STAGE_REDUCE, 1, st);
  dp.launches = launches;
  return DPGB_OK;
}

// the error (if any) that the status words h of an evaluation report
int status_result(DeepPotImpl& dp, const int* h) {
  if (h[kStatusOverflow] > 0)
    return fail(DPGB_EOVERFLOW, "neighbour capacity exceeded (" + std::to_string(h[kStatusOverflow]) +
                                    " entries) at atom/row " + std::to_string(h[kStatusOverflowAtom] - 1));
  if (h[kStatusNonFinite] > 0)
    return fail(DPGB_EINVAL, "non-finite input coordinate (atom " + std::to_string(h[kStatusNonFinite] - 1) +
                                 "); results are invalid");
  if (h[kStatusTimeout] > 0)
    return fail(DPGB_ETIMEOUT, "a tensor-core completion wait timed out; results are invalid");
  if (h[kStatusTruncated] > 0) {
    dp.skin_grow = h[kStatusTruncated];  // the next call widens the candidate rows and rebuilds
    return fail(DPGB_EOVERFLOW, "skin candidate rows too narrow (a row needs " + std::to_string(h[kStatusTruncated]) +
                                    " slots within rcut + skin); results are invalid");
  }
  return DPGB_OK;
}

int check_status(DeepPotImpl& dp, cudaStream_t st) {
  int h[kStatusSlots];
  DPGB_TRY(read_status(dp.ws_status.as<int>(), st, h));
  return status_result(dp, h);
}

// ---- the descriptor stage on its own (mixed form) -------------------------

// out[row] = in[row_pos[row]] over dim values (typed rows; a virtual row is zero)
__global__ void unsort_rows_kernel(float* __restrict__ out, const float* __restrict__ in, const int* __restrict__ row_pos,
                                   const int* __restrict__ atype, int nloc, long long total, int dim) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= total) return;
  const long long row = q / dim;
  const int k = (int)(q - row * dim);
  out[q] = atype[row % nloc] < 0 ? 0.f : in[(size_t)row_pos[row] * dim + k];
}
// out[row_pos[row]] = in[row]
__global__ void sort_rows_kernel(float* __restrict__ out, const float* __restrict__ in, const int* __restrict__ row_pos,
                                 const int* __restrict__ atype, int nloc, long long total, int dim) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= total) return;
  const long long row = q / dim;
  const int k = (int)(q - row * dim);
  if (atype[row % nloc] >= 0) out[(size_t)row_pos[row] * dim + k] = in[q];
}
// transpose keys of a per-frame extended list: frame f's atom nb -> f * nall + nb
__global__ void ext_keys_kernel(int* __restrict__ keys, const int* __restrict__ nlist, long long npair, FastDiv by_row,
                                int nloc, int nall) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npair) return;
  const int nb = nlist[p];
  const int row = by_row.div((int)p), f = row / nloc;
  keys[p] = nb < 0 ? -1 : f * nall + nb;
}
// dE/dr of every extended atom from the pair gradients g = dE/d(r_nb - r_i):
// -sum over the atom's own real slots (local atoms) + sum over the pairs
// that point at it, in FP64 in a fixed order
__global__ void ext_pair_gather_kernel(double* __restrict__ out, const float* __restrict__ g,
                                       const int* __restrict__ nlist, Transpose tr, int nloc, int nall, int nnei,
                                       int nf) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= (long long)nf * nall) return;
  const int f = (int)(q / nall), j = (int)(q - (long long)f * nall);
  double acc[3] = {0.0, 0.0, 0.0};
  if (j < nloc) {
    const size_t row = (size_t)f * nloc + j;
    for (int s = 0; s < nnei; ++s)
      if (nlist[row * nnei + s] >= 0)
#pragma unroll
        for (int k = 0; k < 3; ++k) acc[k] -= (double)g[(row * nnei + s) * 3 + k];
  }
  for (int t = tr.offsets[q]; t < tr.offsets[q + 1]; ++t) {
    const int p = tr.pairs[t];
#pragma unroll
    for (int k = 0; k < 3; ++k) acc[k] += (double)g[3 * (size_t)p + k];
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) out[3 * q + k] = acc[k];
}

// The embedding stage of the mixed form behind DescrptSeA: D (FP32, rows in
// frame-major order) and xyz = G^T R~ / nnei from per-frame extended
// coordinates and a formatted list (typed sections, -1 padding) — the same
// kernels as the full evaluation (tensor-core embedding, or the fused table
// kernels of a compressed model).  The backward turns dE/dD into dE/dr of
// every extended atom.  The forward's state stays in the handle until the
// next forward.
int descrpt_fwd(DeepPotImpl& dp, int nf, int nloc, int nall, const double* coord_ext, const int* atype_ext,
                const int* atype_loc_host, const int* nlist_in, float* D_out, float* xyz_out, cudaStream_t st) {
  if (dp.precision != DPGB_PREC_MIXED)
    return fail(DPGB_EINVAL, "the descriptor stage on its own runs in the mixed form only");
  if (!dp.use_tc && !dp.use_tab)
    return fail(DPGB_EINVAL, "no tensor-core embedding for these embedding widths (and no tables)");
  if (nf < 1 || nloc < 1 || nall < nloc || !coord_ext || !atype_ext || !atype_loc_host || !nlist_in || !D_out)
    return fail(DPGB_EINVAL, "descrpt: bad arguments");
  const dpgb_se_a_desc& d = dp.desc;
  const int nnei = dp.sel.nnei, ng = dp.ng, dim = dp.dim;
  const long long nrows = (long long)nf * nloc, npair = nrows * nnei;
  if (npair >= (1LL << 31) || (long long)nf * nall >= (1LL << 31)) return fail(DPGB_EINVAL, "descrpt: too large");
  dp.dm_eval = 0;
  const unsigned long long eval_no = ++dp.evals;
  DPGB_TRY(prepare_types(dp, nf, nloc, atype_loc_host, st));
  DevModel<float>& m = *dp.m32;
  DPGB_TRY(dp.ws_status.alloc(sizeof(int) * kStatusSlots));
  DPGB_TRY(dp.ws_nlist.alloc(sizeof(int) * npair));
  DPGB_TRY(dp.ws_xyz.alloc(sizeof(float) * nrows * 4 * ng));
  DPGB_TRY(dp.ws_D.alloc(sizeof(float) * nrows * dim));
  DPGB_TRY(dp.ws_dD.alloc(sizeof(float) * nrows * dim));
  DPGB_TRY(dp.ws_g.alloc(sizeof(float) * npair * 3));
  DPGB_TRY(dp.ws_vir.alloc(sizeof(double) * nrows * 9));
  DPGB_TRY(dp.ws_xhi.alloc(sizeof(float4) * (size_t)nf * nall));
  DPGB_TRY(dp.ws_xlo.alloc(sizeof(float4) * (size_t)nf * nall));
  DPGB_TRY(dp.ws_dxyz.alloc(sizeof(float) * nrows * 4 * ((ng + 15) / 16 * 16) * std::max(d.ntypes, 1)));
  int* status = dp.ws_status.as<int>();
  DPGB_CUDA(cudaMemsetAsync(status, 0, sizeof(int) * kStatusSlots, st));
  DPGB_CUDA(cudaMemcpyAsync(dp.ws_nlist.ptr, nlist_in, sizeof(int) * npair, cudaMemcpyDeviceToDevice, st));
  split_points_kernel<<<ceil_div((long long)nf * nall, 256), 256, 0, st>>>(dp.ws_xhi.as<float4>(),
                                                                          dp.ws_xlo.as<float4>(), coord_ext, nf * nall);
  DPGB_TRY(check_launch("split_points"));
  DescParams<float> p{};
  p.nloc = nloc;
  p.nrows = (int)nrows;
  p.nnei = nnei;
  p.ntypes = d.ntypes;
  for (int t = 0; t <= d.ntypes; ++t) p.sec[t] = dp.sel.sec[t];
  p.type_one_side = d.type_one_side;
  p.ng = ng;
  p.axis = d.axis_neuron;
  p.pad_zero = dp.pad_zero;
  p.rcut = d.rcut;
  p.rcut_smth = d.rcut_smth;
  p.davg = m.davg;
  p.dstd = m.dstd;
  p.dstd_inv = m.dstd_inv;
  p.nloc_div = FastDiv(nloc);
  p.pair_mask = d.pair_mask ? dp.pair_mask_dev.as<int>() : nullptr;
  p.atype = dp.atype_dev.as<int>();
  p.nlist = dp.ws_nlist.as<int>();
  p.row_pos = dp.row_pos_dev.as<int>();
  p.coord_ext = coord_ext;
  p.atype_ext = atype_ext;
  p.nall = nall;
  p.xhi = dp.ws_xhi.as<float4>();
  p.xlo = dp.ws_xlo.as<float4>();
  if (dp.use_tc) {
    const int nsorted = dp.type_off[d.ntypes];
    DPGB_TRY(dp.ws_runlen.alloc(sizeof(int) * (size_t)std::max(nsorted, 1) * d.ntypes));
    DPGB_TRY(launch_run_lengths(dp.ws_runlen.as<int>(), p.nlist, dp.sorted_rows_dev.as<int>(), nsorted, nnei, dp.sel,
                                dp.pad_zero, st));
    EmbTC e = dp.tc;
    e.d_bf16 = 0;
    DPGB_TRY(launch_emb_tc_fwd(p, e, dp.chunks_dev.as<WorkChunk>(), dp.nchunks, dp.ws_runlen.as<int>(),
                               dp.sorted_rows_dev.as<int>(), dp.ws_xyz.as<float>(), dp.ws_dxyz.as<float>(),
                               dp.ws_D.as<float>(), status, st));
  } else {
    DPGB_TRY(dp.ws_env.alloc(sizeof(float4) * 2 * npair));
    DPGB_TRY(launch_tab_fwd(p, m.emb, dp.chunks_dev.as<WorkChunk>(), dp.nchunks, dp.sorted_rows_dev.as<int>(),
                            dp.ws_xyz.as<float>(), dp.ws_D.ptr, 0, st, nullptr, dp.ws_env.as<float4>()));
  }
  const long long tot = nrows * dim;
  unsort_rows_kernel<<<ceil_div(tot, 256), 256, 0, st>>>(D_out, dp.ws_D.as<float>(), p.row_pos, p.atype, nloc, tot,
                                                         dim);
  DPGB_TRY(check_launch("unsort_rows"));
  if (xyz_out)
    DPGB_CUDA(cudaMemcpyAsync(xyz_out, dp.ws_xyz.ptr, sizeof(float) * nrows * 4 * ng, cudaMemcpyDeviceToDevice, st));
  dp.dm_p = p;
  dp.dm_nf = nf;
  dp.dm_nloc = nloc;
  dp.dm_nall = nall;
  dp.dm_eval = eval_no;
  return DPGB_OK;
}

int descrpt_bwd(DeepPotImpl& dp, unsigned long long ticket, const float* dD_in, double* g_ext, cudaStream_t st) {
  if (!dD_in || !g_ext) return fail(DPGB_EINVAL, "descrpt_bwd: NULL argument");
  if (!dp.dm_eval || dp.dm_eval != dp.evals || ticket != dp.dm_eval)
    return fail(DPGB_EINVAL, "descrpt_bwd: no descriptor forward of this handle to differentiate (another "
                             "evaluation ran in between)");
  const DescParams<float>& p = dp.dm_p;
  const int nf = dp.dm_nf, nloc = dp.dm_nloc, nall = dp.dm_nall, nnei = p.nnei, dim = dp.dim;
  const long long nrows = (long long)nf * nloc, npair = nrows * nnei, nkeys = (long long)nf * nall;
  int* status = dp.ws_status.as<int>();
  const long long tot = nrows * dim;
  sort_rows_kernel<<<ceil_div(tot, 256), 256, 0, st>>>(dp.ws_dD.as<float>(), dD_in, p.row_pos, p.atype, nloc, tot, dim);
  DPGB_TRY(check_launch("sort_rows"));
  DPGB_CUDA(cudaMemsetAsync(dp.ws_vir.ptr, 0, sizeof(double) * nrows * 9, st));
  DPGB_CUDA(cudaMemsetAsync(dp.ws_g.ptr, 0, sizeof(float) * npair * 3, st));  // slots no kernel visits add 0
  DPGB_TRY(launch_dxyz(p, dp.ws_dD.as<float>(), dp.ws_xyz.as<float>(), dp.ws_dxyz.as<float>(), st));
  if (dp.use_tc)
    DPGB_TRY(launch_emb_tc_bwd(p, dp.tc, dp.chunks_dev.as<WorkChunk>(), dp.nchunks, dp.ws_runlen.as<int>(),
                               dp.sorted_rows_dev.as<int>(), dp.ws_dxyz.as<float>(), dp.ws_g.as<float>(),
                               dp.ws_vir.as<double>(), status, st));
  else
    DPGB_TRY(launch_tab_bwd(p, dp.m32->emb, dp.chunks_dev.as<WorkChunk>(), dp.nchunks, dp.sorted_rows_dev.as<int>(),
                            dp.ws_dxyz.as<float>(), dp.ws_g.as<float>(), dp.ws_vir.as<double>(), st, nullptr,
                            dp.ws_env.as<float4>()));
  DPGB_TRY(dp.dm_keys.alloc(sizeof(int) * npair));
  DPGB_TRY(dp.dm_tr.alloc(transpose_workspace(npair, (int)nkeys)));
  ext_keys_kernel<<<ceil_div(npair, 256), 256, 0, st>>>(dp.dm_keys.as<int>(), p.nlist, npair, FastDiv(nnei), nloc,
                                                        nall);
  DPGB_TRY(check_launch("ext_keys"));
  Transpose tr;
  DPGB_TRY(launch_transpose(tr, dp.dm_keys.as<int>(), npair, (int)nkeys, 0, dp.dm_tr.ptr, status, st));
  ext_pair_gather_kernel<<<ceil_div(nkeys, 256), 256, 0, st>>>(g_ext, dp.ws_g.as<float>(), p.nlist, tr, nloc, nall,
                                                               nnei, nf);
  DPGB_TRY(check_launch("ext_pair_gather"));
  return DPGB_OK;
}

int run_any(DeepPotImpl& dp, int nframes, int natom, const double* coord, const double* box_host, double* energy,
            double* force, double* virial, double* atom_energy, double* atom_virial, cudaStream_t st) {
  if (dp.precision == DPGB_PREC_FP64)
    return run<double>(dp, *dp.m64, nframes, natom, coord, box_host, energy, force, virial, atom_energy, atom_virial, st);
  return run<float>(dp, *dp.m32, nframes, natom, coord, box_host, energy, force, virial, atom_energy, atom_virial, st);
}

int compute_device_impl(DeepPotImpl& dp, int nframes, int natom, const double* coord, const int* atype_host,
                        const double* box_host, double* energy, double* force, double* virial, double* atom_energy,
                        double* atom_virial, cudaStream_t st) {
  if (nframes <= 0 || natom <= 0) return fail(DPGB_EINVAL, "nframes and natom must be positive");
  if (!coord || !atype_host || !energy || !force || !virial) return fail(DPGB_EINVAL, "NULL argument");
  const bool graph = dp.use_graph && box_host && dp.stream;
  const void* ptrs[6] = {coord, energy, force, virial, atom_energy, atom_virial};
  if (graph) {
    DPGB_TRY(prepare_types(dp, nframes, natom, atype_host, st));  // a change of types bumps gen
    const bool same = dp.sg_exec && dp.gen == dp.sg_gen && dp.sg_nframes == nframes && dp.sg_natom == natom &&
                      std::equal(ptrs, ptrs + 6, dp.sg_ptr) &&
                      std::equal(box_host, box_host + 9 * (size_t)nframes, dp.sg_box.begin());
    if (same) {  // replay on the handle's stream, ordered after and before the caller's
      cudaStream_t hs = dp.stream;
      if (st != hs) {
        DPGB_CUDA(cudaEventRecord(dp.sg_ev_in, st));
        DPGB_CUDA(cudaStreamWaitEvent(hs, dp.sg_ev_in, 0));
      }
      DPGB_CUDA(cudaGraphLaunch(dp.sg_exec, hs));
      if (st != hs) {
        DPGB_CUDA(cudaEventRecord(dp.sg_ev_out, hs));
        DPGB_CUDA(cudaStreamWaitEvent(st, dp.sg_ev_out, 0));
      }
      dp.launches = dp.sg_launches;
      return DPGB_OK;
    }
  }
  ++dp.gen;  // workspace may grow
  DPGB_TRY(prepare_types(dp, nframes, natom, atype_host, st));
  DPGB_TRY(run_any(dp, nframes, natom, coord, box_host, energy, force, virial, atom_energy, atom_virial, st));
  if (!graph) return DPGB_OK;
  // capture the same evaluation for the next calls (this call's results come
  // from the plain run; the capture records and does not execute)
  dp.drop_graph();
  if (!dp.sg_ev_in) DPGB_CUDA(cudaEventCreateWithFlags(&dp.sg_ev_in, cudaEventDisableTiming));
  if (!dp.sg_ev_out) DPGB_CUDA(cudaEventCreateWithFlags(&dp.sg_ev_out, cudaEventDisableTiming));
  const int launches = dp.launches, prof = dp.profiling;
  dp.profiling = 0;  // no event records inside the graph
  dp.capturing = 1;
  DPGB_CUDA(cudaStreamBeginCapture(dp.stream, cudaStreamCaptureModeRelaxed));
  const int rc = run_any(dp, nframes, natom, coord, box_host, energy, force, virial, atom_energy, atom_virial,
                         dp.stream);
  cudaGraph_t g = nullptr;
  const cudaError_t ce = cudaStreamEndCapture(dp.stream, &g);
  dp.capturing = 0;
  dp.profiling = prof;
  dp.launches = launches;
  if (rc != DPGB_OK) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  DPGB_CUDA(ce);
  dp.sg_graph = g;
  DPGB_CUDA(cudaGraphInstantiate(&dp.sg_exec, dp.sg_graph, 0));
  dp.sg_gen = dp.gen;
  dp.sg_nframes = nframes;
  dp.sg_natom = natom;
  dp.sg_launches = launches;
  std::copy(ptrs, ptrs + 6, dp.sg_ptr);
  dp.sg_box.assign(box_host, box_host + 9 * (size_t)nframes);
  return DPGB_OK;
}

// One frame with explicit ghosts and a caller's neighbour list (the
// DeepPot::compute(..., nghost, InputNlist, ago) path of
// source/api_cc/src/DeepPotPT.cc:170-243).  ago == 0 (or a changed atom
// count) takes the list afresh; ago > 0 reuses the stored one with the new
// coordinates (the list is re-filtered at rcut and re-ordered every call,
// as forward_lower does).  All pointers are host arrays.
int compute_nlist_impl(DeepPotImpl& dp, int nall, int nghost, const double* coord, const int* atype, int inum,
                       const int* ilist, const int* numneigh, const int* const* firstneigh, int ago, double* energy,
                       double* force, double* virial, double* atom_energy, double* atom_virial) {
  const int nloc = nall - nghost;
  if (nall <= 0 || nghost < 0 || nloc <= 0) return fail(DPGB_EINVAL, "need nall > nghost >= 0");
  if (!coord || !atype || !energy || !force || !virial) return fail(DPGB_EINVAL, "NULL argument");
  cudaStream_t st = dp.stream;
  ++dp.gen;  // workspace may grow
  const bool fresh = ago == 0 || dp.ext_nloc != nloc || dp.ext_nall != nall;
  if (fresh) {
    if (inum != nloc || !ilist || !numneigh || !firstneigh)
      return fail(DPGB_EINVAL, "a new neighbour list needs inum == nall - nghost and ilist / numneigh / firstneigh");
    std::vector<int> off(nloc + 1, 0), cnt(nloc, -1);
    int maxn = 0;
    for (int ii = 0; ii < inum; ++ii) {
      const int i = ilist[ii];
      if (i < 0 || i >= nloc || cnt[i] >= 0) return fail(DPGB_EINVAL, "ilist must list each local atom once");
      if (numneigh[ii] < 0) return fail(DPGB_EINVAL, "negative numneigh");
      cnt[i] = numneigh[ii];
      maxn = std::max(maxn, numneigh[ii]);
    }
    for (int i = 0; i < nloc; ++i) off[i + 1] = off[i] + cnt[i];
    std::vector<int> idx((size_t)std::max(off[nloc], 1), -1);
    for (int ii = 0; ii < inum; ++ii) {
      const int i = ilist[ii];
      for (int k = 0; k < numneigh[ii]; ++k) {
        const int j = firstneigh[ii][k];
        if (j < 0 || j >= nall) return fail(DPGB_EINVAL, "neighbour index outside [0, nall)");
        idx[(size_t)off[i] + k] = j;
      }
    }
    DPGB_TRY(dp.ext_off.alloc(sizeof(int) * (nloc + 1)));
    DPGB_TRY(dp.ext_idx.alloc(sizeof(int) * idx.size()));
    DPGB_CUDA(cudaMemcpyAsync(dp.ext_off.ptr, off.data(), sizeof(int) * off.size(), cudaMemcpyHostToDevice, st));
    DPGB_CUDA(cudaMemcpyAsync(dp.ext_idx.ptr, idx.data(), sizeof(int) * idx.size(), cudaMemcpyHostToDevice, st));
    // forward_lower sorts (and cuts to sum(sel)) when the rows are wider
    // than sum(sel) or the model is compressed (make_model.py:592-658)
    dp.ext_sorted = (maxn > dp.sel.nnei || dp.desc.compressed) ? 1 : 0;
    dp.ext_nloc = nloc;
    dp.ext_nall = nall;
    DPGB_CUDA(cudaStreamSynchronize(st));  // host staging vectors go out of scope
  }
  if (dp.ext_atype_h.size() != (size_t)nall || !std::equal(atype, atype + nall, dp.ext_atype_h.begin())) {
    dp.ext_atype_h.assign(atype, atype + nall);
    DPGB_TRY(dp.ext_atype.alloc(sizeof(int) * nall));
    DPGB_CUDA(cudaMemcpyAsync(dp.ext_atype.ptr, dp.ext_atype_h.data(), sizeof(int) * nall, cudaMemcpyHostToDevice,
                              st));
  }
  DPGB_TRY(prepare_types(dp, 1, nloc, atype, st));
  DPGB_TRY(dp.io_coord.alloc(sizeof(double) * nall * 3));
  DPGB_TRY(dp.io_force.alloc(sizeof(double) * nall * 3));
  DPGB_TRY(dp.io_e.alloc(sizeof(double)));
  DPGB_TRY(dp.io_v.alloc(sizeof(double) * 9));
  DPGB_TRY(dp.io_ae.alloc(sizeof(double) * nall));
  if (atom_virial) DPGB_TRY(dp.io_av.alloc(sizeof(double) * nall * 9));
  DPGB_CUDA(cudaMemcpyAsync(dp.io_coord.ptr, coord, sizeof(double) * nall * 3, cudaMemcpyHostToDevice, st));
  DPGB_CUDA(cudaMemsetAsync(dp.io_ae.ptr, 0, sizeof(double) * nall, st));  // ghosts carry no atom energy
  ExtList ext{dp.io_coord.as<double>(), dp.ext_atype.as<int>(), nall, dp.ext_off.as<int>(), dp.ext_idx.as<int>(),
              dp.ext_sorted};
  double* ae = dp.io_ae.as<double>();
  double* av = atom_virial ? dp.io_av.as<double>() : nullptr;
  if (dp.precision == DPGB_PREC_FP64)
    DPGB_TRY(run<double>(dp, *dp.m64, 1, nloc, dp.io_coord.as<double>(), nullptr, dp.io_e.as<double>(),
                         dp.io_force.as<double>(), dp.io_v.as<double>(), ae, av, st, &ext));
  else
    DPGB_TRY(run<float>(dp, *dp.m32, 1, nloc, dp.io_coord.as<double>(), nullptr, dp.io_e.as<double>(),
                        dp.io_force.as<double>(), dp.io_v.as<double>(), ae, av, st, &ext));
  DPGB_CUDA(cudaMemcpyAsync(energy, dp.io_e.ptr, sizeof(double), cudaMemcpyDeviceToHost, st));
  DPGB_CUDA(cudaMemcpyAsync(force, dp.io_force.ptr, sizeof(double) * nall * 3, cudaMemcpyDeviceToHost, st));
  DPGB_CUDA(cudaMemcpyAsync(virial, dp.io_v.ptr, sizeof(double) * 9, cudaMemcpyDeviceToHost, st));
  if (atom_energy)
    DPGB_CUDA(cudaMemcpyAsync(atom_energy, dp.io_ae.ptr, sizeof(double) * nall, cudaMemcpyDeviceToHost, st));
  if (atom_virial)
    DPGB_CUDA(cudaMemcpyAsync(atom_virial, dp.io_av.ptr, sizeof(double) * nall * 9, cudaMemcpyDeviceToHost, st));
  return check_status(dp, st);  // synchronises
}

// ---- batches of frames of different sizes ------------------------------------

// cell geometry and image tables of one periodic frame, in the reference's
// image range (nbuff = ceil(rcut / face distance))
int frame_geometry(const double* c, double rcut, CellGeom& g, std::vector<int>& spos, std::vector<double>& svec) {
  auto crn = [&](int p, int q) {
    const double x = c[p * 3 + 1] * c[q * 3 + 2] - c[p * 3 + 2] * c[q * 3 + 1];
    const double y = c[p * 3 + 2] * c[q * 3 + 0] - c[p * 3 + 0] * c[q * 3 + 2];
    const double z = c[p * 3 + 0] * c[q * 3 + 1] - c[p * 3 + 1] * c[q * 3 + 0];
    return std::sqrt(x * x + y * y + z * z);
  };
  const double vol = std::fabs(c[0] * (c[4] * c[8] - c[5] * c[7]) - c[1] * (c[3] * c[8] - c[5] * c[6]) +
                               c[2] * (c[3] * c[7] - c[4] * c[6]));
  if (!(vol > 0)) return fail(DPGB_EINVAL, "batch frame with a degenerate box");
  const int nb[3] = {(int)std::ceil(rcut / (vol / crn(1, 2))), (int)std::ceil(rcut / (vol / crn(2, 0))),
                     (int)std::ceil(rcut / (vol / crn(0, 1)))};
  const std::vector<int> shifts = default_shifts(nb);
  const int ns = (int)shifts.size() / 3;
  DPGB_TRY(periodic_geom(c, rcut, ns, shifts.data(), g, spos));
  for (int k = 0; k < 3; ++k)
    if (g.reach[k] > 2) return fail(DPGB_EINVAL, "batch frame thinner than rcut / 2 across a face");
  shift_vectors(g, shifts.data(), ns, svec);
  return DPGB_OK;
}

struct BatchImpl {
  DeepPotImpl* dp = nullptr;
  int nframes = 0, natoms = 0, ncells = 0;
  std::vector<int> atype, atom_off_h;
  BatchPlan plan;
  int bucket_frames[DPGB_BATCH_BUCKETS] = {}, bucket_atoms[DPGB_BATCH_BUCKETS] = {};
  DeviceBuffer atom_off, cell_off, spos_off, svec_off, geom, svec, spos;
  BatchIn in{};
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  const void* cap_ptr[4] = {};
  cudaStream_t cap_stream = nullptr;
  unsigned long long cap_gen = ~0ull;
  ~BatchImpl() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
  }
};

int batch_setup(BatchImpl& b, DeepPotImpl& dp, int nframes, const int* natoms, const int* atype, const double* box) {
  if (nframes < 1 || !natoms || !atype || !box) return fail(DPGB_EINVAL, "batch: bad arguments");
  b.dp = &dp;
  b.nframes = nframes;
  b.atom_off_h.assign(nframes + 1, 0);
  std::vector<int> cell_off(nframes + 1, 0), spos_off(nframes + 1, 0), svec_off(nframes + 1, 0);
  std::vector<CellGeom> geom(nframes);
  std::vector<int> spos_all;
  std::vector<double> svec_all;
  for (int f = 0; f < nframes; ++f) {
    if (natoms[f] < 1) return fail(DPGB_EINVAL, "batch: a frame without atoms");
    b.atom_off_h[f + 1] = b.atom_off_h[f] + natoms[f];
    std::vector<int> sp;
    std::vector<double> sv;
    DPGB_TRY(frame_geometry(box + 9 * f, dp.desc.rcut, geom[f], sp, sv));
    cell_off[f + 1] = cell_off[f] + geom[f].ncell[0] * geom[f].ncell[1] * geom[f].ncell[2];
    spos_off[f + 1] = spos_off[f] + (int)sp.size();
    svec_off[f + 1] = svec_off[f] + (int)sv.size() / 3;
    spos_all.insert(spos_all.end(), sp.begin(), sp.end());
    svec_all.insert(svec_all.end(), sv.begin(), sv.end());
  }
  b.natoms = b.atom_off_h[nframes];
  b.ncells = cell_off[nframes];
  b.atype.assign(atype, atype + b.natoms);
  b.plan.row_bucket.assign(b.natoms, 0);
  b.plan.version = ++plan_versions;
  for (int f = 0; f < nframes; ++f) {
    const int k = bucket_of(natoms[f]);
    ++b.bucket_frames[k];
    b.bucket_atoms[k] += natoms[f];
    std::fill(b.plan.row_bucket.begin() + b.atom_off_h[f], b.plan.row_bucket.begin() + b.atom_off_h[f + 1], k);
  }
  DPGB_TRY(b.atom_off.alloc(sizeof(int) * (nframes + 1)));
  DPGB_TRY(b.cell_off.alloc(sizeof(int) * (nframes + 1)));
  DPGB_TRY(b.spos_off.alloc(sizeof(int) * (nframes + 1)));
  DPGB_TRY(b.svec_off.alloc(sizeof(int) * (nframes + 1)));
  DPGB_TRY(b.geom.alloc(sizeof(CellGeom) * nframes));
  DPGB_TRY(b.spos.alloc(sizeof(int) * spos_all.size()));
  DPGB_TRY(b.svec.alloc(sizeof(double) * svec_all.size()));
  DPGB_CUDA(cudaMemcpy(b.atom_off.ptr, b.atom_off_h.data(), sizeof(int) * (nframes + 1), cudaMemcpyHostToDevice));
  DPGB_CUDA(cudaMemcpy(b.cell_off.ptr, cell_off.data(), sizeof(int) * (nframes + 1), cudaMemcpyHostToDevice));
  DPGB_CUDA(cudaMemcpy(b.spos_off.ptr, spos_off.data(), sizeof(int) * (nframes + 1), cudaMemcpyHostToDevice));
  DPGB_CUDA(cudaMemcpy(b.svec_off.ptr, svec_off.data(), sizeof(int) * (nframes + 1), cudaMemcpyHostToDevice));
  DPGB_CUDA(cudaMemcpy(b.geom.ptr, geom.data(), sizeof(CellGeom) * nframes, cudaMemcpyHostToDevice));
  DPGB_CUDA(cudaMemcpy(b.spos.ptr, spos_all.data(), sizeof(int) * spos_all.size(), cudaMemcpyHostToDevice));
  DPGB_CUDA(cudaMemcpy(b.svec.ptr, svec_all.data(), sizeof(double) * svec_all.size(), cudaMemcpyHostToDevice));
  b.in.ft = FrameTab{nframes, b.atom_off.as<int>(), b.cell_off.as<int>(), b.spos_off.as<int>(), b.svec_off.as<int>(),
                     b.geom.as<CellGeom>()};
  b.in.ncells = b.ncells;
  b.in.svec = b.svec.as<double>();
  b.in.spos = b.spos.as<int>();
  b.in.max_atoms = *std::max_element(natoms, natoms + nframes);
  b.in.nsvec = (int)(svec_all.size() / 3);
  return DPGB_OK;
}

int batch_run(BatchImpl& b, const double* coord, double* energy, double* force, double* virial, cudaStream_t st) {
  DeepPotImpl& dp = *b.dp;
  if (dp.precision == DPGB_PREC_FP64)
    return run<double>(dp, *dp.m64, 1, b.natoms, coord, nullptr, energy, force, virial, nullptr, nullptr, st, nullptr,
                       &b.in);
  return run<float>(dp, *dp.m32, 1, b.natoms, coord, nullptr, energy, force, virial, nullptr, nullptr, st, nullptr,
                    &b.in);
}

// Device coordinates in, device outputs; with use_graph the kernel sequence
// is captured once (after one plain evaluation has sized every buffer) and
// replayed while the handle's cached state and the buffers stay the same.
int batch_compute(BatchImpl& b, const double* coord, double* energy, double* force, double* virial,
                  cudaStream_t st, int use_graph) {
  DeepPotImpl& dp = *b.dp;
  if (!coord || !energy || !force || !virial) return fail(DPGB_EINVAL, "batch: NULL argument");
  DPGB_TRY(prepare_types(dp, 1, b.natoms, b.atype.data(), st, &b.plan));
  const void* ptrs[4] = {coord, energy, force, virial};
  const bool same = b.exec && dp.gen == b.cap_gen && st == b.cap_stream &&
                    std::equal(ptrs, ptrs + 4, b.cap_ptr);
  if (use_graph && same) {
    DPGB_CUDA(cudaGraphLaunch(b.exec, st));
    return DPGB_OK;
  }
  DPGB_TRY(batch_run(b, coord, energy, force, virial, st));
  if (!use_graph) return DPGB_OK;
  if (b.exec) {
    cudaGraphExecDestroy(b.exec);
    b.exec = nullptr;
  }
  if (b.graph) {
    cudaGraphDestroy(b.graph);
    b.graph = nullptr;
  }
  const int prof = dp.profiling;
  dp.profiling = 0;  // no event records inside the graph
  DPGB_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed));
  const int rc = batch_run(b, coord, energy, force, virial, st);
  cudaGraph_t g = nullptr;
  const cudaError_t ce = cudaStreamEndCapture(st, &g);
  dp.profiling = prof;
  DPGB_TRY(rc);
  DPGB_CUDA(ce);
  b.graph = g;
  DPGB_CUDA(cudaGraphInstantiate(&b.exec, b.graph, 0));
  std::copy(ptrs, ptrs + 4, b.cap_ptr);
  b.cap_gen = dp.gen;
  b.cap_stream = st;
  return DPGB_OK;
}

}  // namespace
}  // namespace dpgb

using namespace dpgb;

struct dpgb_deeppot {
  DeepPotImpl impl;
};

namespace dpgb {
namespace {
// record the completion of an evaluation issued on st
int mark_done(DeepPotImpl& im, cudaStream_t st) {
  if (!im.last_done) DPGB_CUDA(cudaEventCreateWithFlags(&im.last_done, cudaEventDisableTiming));
  DPGB_CUDA(cudaEventRecord(im.last_done, st));
  return DPGB_OK;
}
}  // namespace
}  // namespace dpgb

extern "C" {

dpgb_deeppot* dpgb_deeppot_new(const dpgb_se_a_desc* desc, int precision) {
  clear_error();
  if (validate_desc(desc) != DPGB_OK) return nullptr;
  if (precision != DPGB_PREC_FP64 && precision != DPGB_PREC_MIXED) {
    fail(DPGB_EINVAL, "unknown precision");
    return nullptr;
  }
  std::unique_ptr<dpgb_deeppot> dp(new dpgb_deeppot());
  DeepPotImpl& im = dp->impl;
  im.desc = *desc;
  im.precision = precision;
  if (sel_from_host(desc->sel, desc->ntypes, im.sel) != DPGB_OK) return nullptr;
  im.ng = desc->emb_neuron[desc->n_emb - 1];
  im.dim = desc->dim_descrpt;
  im.nnets = desc->type_one_side ? desc->ntypes : desc->ntypes * desc->ntypes;
  im.pad_zero = 1;
  for (size_t q = 0; q < (size_t)desc->ntypes * im.sel.nnei * 4; ++q)
    if (desc->davg[q] != 0.0) im.pad_zero = 0;
  std::vector<double> bias(desc->atom_ener_bias, desc->atom_ener_bias + desc->ntypes);
  if (im.bias_dev.alloc(sizeof(double) * bias.size()) != DPGB_OK) return nullptr;
  if (cudaMemcpy(im.bias_dev.ptr, bias.data(), sizeof(double) * bias.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
    fail(DPGB_ECUDA, "bias upload failed");
    return nullptr;
  }
  if (desc->pair_mask) {
    if (im.pair_mask_dev.alloc(sizeof(int) * desc->ntypes * desc->ntypes) != DPGB_OK) return nullptr;
    cudaMemcpy(im.pair_mask_dev.ptr, desc->pair_mask, sizeof(int) * desc->ntypes * desc->ntypes, cudaMemcpyHostToDevice);
  }
  if (precision == DPGB_PREC_FP64) {
    im.m64.reset(new DevModel<double>());
    if (build_dev_model<double>(im, *im.m64) != DPGB_OK) return nullptr;
  } else {
    im.m32.reset(new DevModel<float>());
    if (build_dev_model<float>(im, *im.m32) != DPGB_OK) return nullptr;
    const char* no_tc = getenv("DPGB_NO_TENSOR_CORES");
    if (emb_tc_eligible(*desc) && !(no_tc && no_tc[0] == '1')) {
      std::vector<unsigned char> img;
      std::vector<float> vec;
      if (build_emb_tc(*desc, img, im.tc, vec) != DPGB_OK) return nullptr;
      if (im.tc_images.alloc(img.size()) != DPGB_OK || im.tc_vec.alloc(sizeof(float) * vec.size()) != DPGB_OK)
        return nullptr;
      if (cudaMemcpy(im.tc_images.ptr, img.data(), img.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
          cudaMemcpy(im.tc_vec.ptr, vec.data(), sizeof(float) * vec.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
        fail(DPGB_ECUDA, "tensor-core weight upload failed");
        return nullptr;
      }
      emb_tc_bind(im.tc, im.tc_images.as<unsigned char>(), 0, im.tc_vec.as<float>());
      im.use_tc = 1;
      if (fit_tc_eligible(*desc) && build_fit_tc(im, *desc) != DPGB_OK) return nullptr;
    } else if (desc->compressed && tab_fused_eligible(im.ng, desc->axis_neuron) && !(no_tc && no_tc[0] == '1')) {
      // compressed nets: fused FP32 table kernels, tensor-core fitting
      im.use_tab = 1;
      if (fit_tc_eligible(*desc) && build_fit_tc(im, *desc) != DPGB_OK) return nullptr;
    }
  }
  // the host pointers of the description are not kept
  for (int e = 0; e < DPGB_MAX_TYPES * DPGB_MAX_TYPES; ++e) {
    for (int l = 0; l < DPGB_MAX_LAYERS; ++l) im.desc.emb_w[e][l] = im.desc.emb_b[e][l] = im.desc.emb_idt[e][l] = nullptr;
    im.desc.table[e] = nullptr;
  }
  for (int t = 0; t < DPGB_MAX_TYPES; ++t)
    for (int l = 0; l <= DPGB_MAX_LAYERS; ++l) im.desc.fit_w[t][l] = im.desc.fit_b[t][l] = im.desc.fit_idt[t][l] = nullptr;
  im.desc.davg = im.desc.dstd = im.desc.atom_ener_bias = nullptr;
  if (cudaStreamCreateWithFlags(&im.stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&im.side, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&im.ev_fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&im.ev_join, cudaEventDisableTiming) != cudaSuccess) {
    fail(DPGB_ECUDA, "stream creation failed");
    return nullptr;
  }
  return dp.release();
}

void dpgb_deeppot_delete(dpgb_deeppot* dp) {
  if (!dp) return;
  if (dp->impl.stream) {
    cudaStreamSynchronize(dp->impl.stream);
    cudaStreamDestroy(dp->impl.stream);
  }
  for (auto& e : dp->impl.ev)
    if (e) cudaEventDestroy(e);
  dp->impl.drop_graph();
  if (dp->impl.side) {
    cudaStreamSynchronize(dp->impl.side);
    cudaStreamDestroy(dp->impl.side);
  }
  if (dp->impl.ev_fork) cudaEventDestroy(dp->impl.ev_fork);
  if (dp->impl.ev_join) cudaEventDestroy(dp->impl.ev_join);
  if (dp->impl.sg_ev_in) cudaEventDestroy(dp->impl.sg_ev_in);
  if (dp->impl.sg_ev_out) cudaEventDestroy(dp->impl.sg_ev_out);
  if (dp->impl.last_done) {
    cudaEventSynchronize(dp->impl.last_done);
    cudaEventDestroy(dp->impl.last_done);
  }
  delete dp;
}

const char* dpgb_deeppot_check_ok(dpgb_deeppot* dp) { return dp ? dp->impl.err.c_str() : "NULL handle"; }

int dpgb_deeppot_last_launches(dpgb_deeppot* dp) { return dp ? dp->impl.launches : 0; }

int dpgb_deeppot_last_nlist(dpgb_deeppot* dp, int* info, int* nlist, double* coord, double* shift) {
  clear_error();
  if (!dp || !info) return fail(DPGB_EINVAL, "NULL handle or info");
  DeepPotImpl& im = dp->impl;
  info[0] = im.nl_nframes;
  info[1] = im.nl_natom;
  info[2] = im.sel.nnei;
  info[3] = im.nl_nshift;
  if (im.nl_nframes <= 0) {
    if (nlist || coord || shift)
      return fail(DPGB_EINVAL, "the last evaluation built no list of its own (none yet, an external list or a batch)");
    return DPGB_OK;
  }
  const size_t nrows = (size_t)im.nl_nframes * im.nl_natom;
  cudaStream_t st = im.stream;
  if (im.last_done) DPGB_CUDA(cudaStreamWaitEvent(st, im.last_done, 0));  // the list is complete
  if (nlist)
    DPGB_CUDA(cudaMemcpyAsync(nlist, im.ws_nlist.ptr, sizeof(int) * nrows * im.sel.nnei, cudaMemcpyDeviceToHost, st));
  if (coord) DPGB_CUDA(cudaMemcpyAsync(coord, im.ws_coord.ptr, sizeof(double) * nrows * 3, cudaMemcpyDeviceToHost, st));
  if (shift)
    DPGB_CUDA(cudaMemcpyAsync(shift, im.ws_svec.ptr, sizeof(double) * 3 * (size_t)im.nl_nshift * im.nl_nframes,
                              cudaMemcpyDeviceToHost, st));
  DPGB_CUDA(cudaStreamSynchronize(st));
  return DPGB_OK;
}

int dpgb_deeppot_descrpt_fwd(dpgb_deeppot* dp, int nf, int nloc, int nall, const double* coord_ext,
                             const int* atype_ext, const int* atype_loc, const int* nlist, float* descrpt,
                             float* xyz, unsigned long long* ticket, void* stream) {
  clear_error();
  if (!dp) return fail(DPGB_EINVAL, "NULL handle");
  int rc = descrpt_fwd(dp->impl, nf, nloc, nall, coord_ext, atype_ext, atype_loc, nlist, descrpt, xyz, as_stream(stream));
  if (rc == DPGB_OK) rc = mark_done(dp->impl, as_stream(stream));
  if (ticket) *ticket = rc == DPGB_OK ? dp->impl.dm_eval : 0;
  dp->impl.err = rc == DPGB_OK ? "" : dpgb_last_error();
  return rc;
}

int dpgb_deeppot_descrpt_bwd(dpgb_deeppot* dp, unsigned long long ticket, const float* g_descrpt,
                             double* g_coord_ext, void* stream) {
  clear_error();
  if (!dp) return fail(DPGB_EINVAL, "NULL handle");
  int rc = descrpt_bwd(dp->impl, ticket, g_descrpt, g_coord_ext, as_stream(stream));
  if (rc == DPGB_OK) rc = mark_done(dp->impl, as_stream(stream));
  dp->impl.err = rc == DPGB_OK ? "" : dpgb_last_error();
  return rc;
}

int dpgb_deeppot_set_profiling(dpgb_deeppot* dp, int on) {
  clear_error();
  if (!dp) return fail(DPGB_EINVAL, "NULL handle");
  DeepPotImpl& im = dp->impl;
  if (on && !im.ev[0])
    for (auto& e : im.ev) DPGB_CUDA(cudaEventCreate(&e));
  im.profiling = on;
  for (auto& x : im.stage_ms) x = 0.0;
  im.stage_calls = 0;
  im.ev_recorded = 0;
  return DPGB_OK;
}

int dpgb_deeppot_collect_stages(dpgb_deeppot* dp) {
  clear_error();
  if (!dp) return fail(DPGB_EINVAL, "NULL handle");
  DeepPotImpl& im = dp->impl;
  if (!im.profiling || !im.ev_recorded) return DPGB_OK;
  DPGB_CUDA(cudaEventSynchronize(im.ev[2 * DPGB_NUM_STAGES - 1]));
  for (int s = 0; s < DPGB_NUM_STAGES; ++s) {
    float ms = 0.f;
    DPGB_CUDA(cudaEventElapsedTime(&ms, im.ev[2 * s], im.ev[2 * s + 1]));
    im.stage_ms[s] += ms;
  }
  im.stage_calls += 1;
  im.ev_recorded = 0;
  return DPGB_OK;
}

int dpgb_deeppot_stage_times(dpgb_deeppot* dp, double* ms, int* ncalls) {
  clear_error();
  if (!dp || !ms) return fail(DPGB_EINVAL, "NULL argument");
  for (int s = 0; s < DPGB_NUM_STAGES; ++s) ms[s] = dp->impl.stage_ms[s];
  if (ncalls) *ncalls = dp->impl.stage_calls;
  return DPGB_OK;
}

int dpgb_deeppot_compute_device(dpgb_deeppot* dp, int nframes, int natom, const double* coord, const int* atype_host,
                                const double* box_host, double* energy, double* force, double* virial,
                                double* atom_energy, double* atom_virial, void* stream) {
  clear_error();
  if (!dp) return fail(DPGB_EINVAL, "NULL handle");
  int rc = compute_device_impl(dp->impl, nframes, natom, coord, atype_host, box_host, energy, force, virial,
                               atom_energy, atom_virial, as_stream(stream));
  if (rc == DPGB_OK) rc = mark_done(dp->impl, as_stream(stream));
  dp->impl.err = rc == DPGB_OK ? "" : dpgb_last_error();
  return rc;
}

struct dpgb_batch {
  BatchImpl impl;
  dpgb_deeppot* owner = nullptr;
  DeviceBuffer io_c, io_e, io_f, io_v;
};

dpgb_batch* dpgb_batch_new(dpgb_deeppot* dp, int nframes, const int* natoms, const int* atype, const double* box) {
  clear_error();
  if (!dp) {
    fail(DPGB_EINVAL, "NULL handle");
    return nullptr;
  }
  std::unique_ptr<dpgb_batch> b(new dpgb_batch());
  b->owner = dp;
  if (batch_setup(b->impl, dp->impl, nframes, natoms, atype, box) != DPGB_OK) return nullptr;
  return b.release();
}

void dpgb_batch_delete(dpgb_batch* b) { delete b; }

int dpgb_batch_natoms(const dpgb_batch* b) { return b ? b->impl.natoms : -1; }

int dpgb_batch_buckets(const dpgb_batch* b, int* frames, int* atoms) {
  if (!b) return fail(DPGB_EINVAL, "batch: NULL handle");
  for (int k = 0; k < DPGB_BATCH_BUCKETS; ++k) {
    if (frames) frames[k] = b->impl.bucket_frames[k];
    if (atoms) atoms[k] = b->impl.bucket_atoms[k];
  }
  return DPGB_OK;
}

int dpgb_batch_set_tiles(dpgb_batch* b, const int* rows_per_item) {
  if (!b || !rows_per_item) return fail(DPGB_EINVAL, "batch: NULL argument");
  for (int k = 0; k < DPGB_BATCH_BUCKETS; ++k)
    if (rows_per_item[k] < 0 || rows_per_item[k] > (1 << 20)) return fail(DPGB_EINVAL, "batch: tile rows out of range");
  BatchPlan& p = b->impl.plan;
  if (std::equal(rows_per_item, rows_per_item + DPGB_BATCH_BUCKETS, p.tile_rows)) return DPGB_OK;
  std::copy(rows_per_item, rows_per_item + DPGB_BATCH_BUCKETS, p.tile_rows);
  p.version = ++plan_versions;  // the next evaluation re-cuts the items (and re-captures its graph)
  return DPGB_OK;
}

int dpgb_batch_get_tiles(const dpgb_batch* b, int* rows_per_item) {
  if (!b || !rows_per_item) return fail(DPGB_EINVAL, "batch: NULL argument");
  std::copy(b->impl.plan.tile_rows, b->impl.plan.tile_rows + DPGB_BATCH_BUCKETS, rows_per_item);
  return DPGB_OK;
}

int dpgb_batch_compute_device(dpgb_batch* b, const double* coord, double* energy, double* force, double* virial,
                              void* stream, int use_graph) {
  clear_error();
  if (!b) return fail(DPGB_EINVAL, "NULL batch");
  cudaStream_t st = as_stream(stream);
  if (!st) st = b->owner->impl.stream;  // graphs cannot be captured on the legacy stream
  int rc = batch_compute(b->impl, coord, energy, force, virial, st, use_graph);
  if (rc == DPGB_OK) rc = mark_done(b->owner->impl, st);
  if (rc == DPGB_OK && !stream) rc = check_cuda(cudaStreamSynchronize(st), "batch");
  b->owner->impl.err = rc == DPGB_OK ? "" : dpgb_last_error();
  return rc;
}

int dpgb_batch_compute(dpgb_batch* b, const double* coord, double* energy, double* force, double* virial,
                       int use_graph) {
  clear_error();
  if (!b) return fail(DPGB_EINVAL, "NULL batch");
  DeepPotImpl& im = b->owner->impl;
  cudaStream_t st = im.stream;
  auto body = [&]() -> int {
    if (!coord || !energy || !force || !virial) return fail(DPGB_EINVAL, "NULL argument");
    const size_t n = (size_t)b->impl.natoms, nf = (size_t)b->impl.nframes;
    DPGB_TRY(b->io_c.alloc(sizeof(double) * n * 3));
    DPGB_TRY(b->io_f.alloc(sizeof(double) * n * 3));
    DPGB_TRY(b->io_e.alloc(sizeof(double) * nf));
    DPGB_TRY(b->io_v.alloc(sizeof(double) * nf * 9));
    DPGB_CUDA(cudaMemcpyAsync(b->io_c.ptr, coord, sizeof(double) * n * 3, cudaMemcpyHostToDevice, st));
    DPGB_TRY(batch_compute(b->impl, b->io_c.as<double>(), b->io_e.as<double>(), b->io_f.as<double>(),
                           b->io_v.as<double>(), st, use_graph));
    DPGB_CUDA(cudaMemcpyAsync(energy, b->io_e.ptr, sizeof(double) * nf, cudaMemcpyDeviceToHost, st));
    DPGB_CUDA(cudaMemcpyAsync(force, b->io_f.ptr, sizeof(double) * n * 3, cudaMemcpyDeviceToHost, st));
    DPGB_CUDA(cudaMemcpyAsync(virial, b->io_v.ptr, sizeof(double) * nf * 9, cudaMemcpyDeviceToHost, st));
    return check_status(im, st);  // synchronises
  };
  int rc = body();
  im.err = rc == DPGB_OK ? "" : dpgb_last_error();
  return rc;
}

int dpgb_deeppot_compute_nlist(dpgb_deeppot* dp, int nall, int nghost, const double* coord, const int* atype,
                               const double* box, int inum, const int* ilist, const int* numneigh,
                               const int* const* firstneigh, int ago, double* energy, double* force, double* virial,
                               double* atom_energy, double* atom_virial) {
  clear_error();
  if (!dp) return fail(DPGB_EINVAL, "NULL handle");
  (void)box;  // the caller's list and ghost coordinates already encode the periodicity
  int rc = coord && nall > 0 ? check_finite(coord, (size_t)nall * 3, "coordinate") : DPGB_OK;
  if (rc == DPGB_OK)
    rc = compute_nlist_impl(dp->impl, nall, nghost, coord, atype, inum, ilist, numneigh, firstneigh, ago, energy,
                              force, virial, atom_energy, atom_virial);
  dp->impl.err = rc == DPGB_OK ? "" : dpgb_last_error();
  return rc;
}

int dpgb_deeppot_compute(dpgb_deeppot* dp, int nframes, int natom, const double* coord, const int* atype,
                         const double* box, double* energy, double* force, double* virial, double* atom_energy,
                         double* atom_virial) {
  clear_error();
  if (!dp) return fail(DPGB_EINVAL, "NULL handle");
  DeepPotImpl& im = dp->impl;
  cudaStream_t st = im.stream;
  auto body = [&]() -> int {
    if (nframes <= 0 || natom <= 0 || !coord || !atype || !energy || !force || !virial)
      return fail(DPGB_EINVAL, "bad arguments");
    // the outputs are one device block and the host side goes through one
    // pinned block: one copy in, two copies out (outputs, status words), one
    // synchronisation
    const size_t nrow = (size_t)nframes * natom;
    const size_t n_e = nframes, n_v = 9 * (size_t)nframes, n_f = 3 * nrow, n_ae = atom_energy ? nrow : 0,
                 n_av = atom_virial ? 9 * nrow : 0, n_out = n_e + n_v + n_f + n_ae + n_av;
    DPGB_TRY(im.io_coord.alloc(sizeof(double) * 3 * nrow));
    DPGB_TRY(im.io_out.alloc(sizeof(double) * n_out));
    DPGB_TRY(im.io_host.alloc(sizeof(double) * (3 * nrow + n_out) + sizeof(int) * kStatusSlots));
    double* hc = im.io_host.as<double>();
    double* ho = hc + 3 * nrow;
    int* hs = reinterpret_cast<int*>(ho + n_out);
    // page-locked caller buffers are copied directly; pageable ones go
    // through the pinned staging block
    const bool pin_in = is_pinned(coord);
    const bool pin_out = is_pinned(energy) && is_pinned(force) && is_pinned(virial) &&
                         (!atom_energy || is_pinned(atom_energy)) && (!atom_virial || is_pinned(atom_virial));
    if (!pin_in) std::memcpy(hc, coord, sizeof(double) * 3 * nrow);
    DPGB_CUDA(cudaMemcpyAsync(im.io_coord.ptr, pin_in ? coord : hc, sizeof(double) * 3 * nrow, cudaMemcpyHostToDevice,
                              st));
    double* d = im.io_out.as<double>();
    DPGB_TRY(compute_device_impl(im, nframes, natom, im.io_coord.as<double>(), atype, box, d, d + n_e + n_v, d + n_e,
                                 atom_energy ? d + n_e + n_v + n_f : nullptr,
                                 atom_virial ? d + n_e + n_v + n_f + n_ae : nullptr, st));
    if (pin_out) {
      DPGB_CUDA(cudaMemcpyAsync(energy, d, sizeof(double) * n_e, cudaMemcpyDeviceToHost, st));
      DPGB_CUDA(cudaMemcpyAsync(virial, d + n_e, sizeof(double) * n_v, cudaMemcpyDeviceToHost, st));
      DPGB_CUDA(cudaMemcpyAsync(force, d + n_e + n_v, sizeof(double) * n_f, cudaMemcpyDeviceToHost, st));
      if (atom_energy)
        DPGB_CUDA(cudaMemcpyAsync(atom_energy, d + n_e + n_v + n_f, sizeof(double) * n_ae, cudaMemcpyDeviceToHost, st));
      if (atom_virial)
        DPGB_CUDA(cudaMemcpyAsync(atom_virial, d + n_e + n_v + n_f + n_ae, sizeof(double) * n_av,
                                  cudaMemcpyDeviceToHost, st));
    } else {
      DPGB_CUDA(cudaMemcpyAsync(ho, d, sizeof(double) * n_out, cudaMemcpyDeviceToHost, st));
    }
    DPGB_CUDA(cudaMemcpyAsync(hs, im.ws_status.ptr, sizeof(int) * kStatusSlots, cudaMemcpyDeviceToHost, st));
    DPGB_CUDA(cudaStreamSynchronize(st));
    if (!pin_out) {
      std::memcpy(energy, ho, sizeof(double) * n_e);
      std::memcpy(virial, ho + n_e, sizeof(double) * n_v);
      std::memcpy(force, ho + n_e + n_v, sizeof(double) * n_f);
      if (atom_energy) std::memcpy(atom_energy, ho + n_e + n_v + n_f, sizeof(double) * n_ae);
      if (atom_virial) std::memcpy(atom_virial, ho + n_e + n_v + n_f + n_ae, sizeof(double) * n_av);
    }
    return status_result(im, hs);
  };
  int rc = body();
  if (rc == DPGB_EOVERFLOW && im.skin_grow > 0) rc = body();  // widened skin candidates, rebuilt
  im.err = rc == DPGB_OK ? "" : dpgb_last_error();
  return rc;
}

int dpgb_deeppot_set_skin(dpgb_deeppot* dp, double skin, int every) {
  clear_error();
  if (!dp) return fail(DPGB_EINVAL, "NULL handle");
  if (!(skin >= 0.0) || every < 1) return fail(DPGB_EINVAL, "skin must be >= 0 and every >= 1");
  DeepPotImpl& im = dp->impl;
  im.skin = skin;
  im.skin_every = every;
  im.skin_nframes = -1;  // the next call builds
  return DPGB_OK;
}

int dpgb_deeppot_set_graph(dpgb_deeppot* dp, int on) {
  clear_error();
  if (!dp) return fail(DPGB_EINVAL, "NULL handle");
  dp->impl.use_graph = on ? 1 : 0;
  if (!on) dp->impl.drop_graph();
  return DPGB_OK;
}

int dpgb_deeppot_check_status(dpgb_deeppot* dp, void* stream) {
  clear_error();
  if (!dp) return fail(DPGB_EINVAL, "NULL handle");
  DeepPotImpl& im = dp->impl;
  if (!im.ws_status.ptr) return DPGB_OK;
  cudaStream_t st = as_stream(stream);
  if (!st) {  // the last evaluation's stream, through its completion event
    st = im.stream;
    if (im.last_done) DPGB_CUDA(cudaStreamWaitEvent(st, im.last_done, 0));
  }
  const int rc = check_status(im, st);
  im.err = rc == DPGB_OK ? "" : dpgb_last_error();
  return rc;
}

}  // extern "C"
