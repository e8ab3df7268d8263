// Device-side description of a se_e2_a model and the launchers of the fused
// descriptor / fitting kernels used by the DeepPot pipeline.
#pragma once

#include "nlist.cuh"

namespace dpgb {

constexpr int kMaxEmbLayers = 4;
constexpr int kMaxFitLayers = 5;
constexpr int kMaxNets = DPGB_MAX_TYPES * DPGB_MAX_TYPES;

// Table interval data of one compressed net (locate_xx constants).
template <typename T>
struct TabMeta {
  T lower, upper, mx, s0, s1, hi_xx;
  int first, hi_idx;
  long long offset;  // element offset of the net's table in the table buffer
};

// Quintic of one table interval and its derivative; delta != 0 extends the
// end intervals linearly (tabulate.cc locate_xx_se_a with extrapolation).
template <typename T>
__device__ __forceinline__ void table_poly(const T* rowc, T xx, T delta, T& val, T& grad) {
  const T a0 = rowc[0], a1 = rowc[1], a2 = rowc[2], a3 = rowc[3], a4 = rowc[4], a5 = rowc[5];
  grad = a1 + ((T)2 * a2 + ((T)3 * a3 + ((T)4 * a4 + (T)5 * a5 * xx) * xx) * xx) * xx;
  val = a0 + (a1 + (a2 + (a3 + (a4 + a5 * xx) * xx) * xx) * xx) * xx + grad * delta;
}

// interval index and offset of x (source/lib/src/tabulate.cc locate_xx_se_a)
template <typename T>
__device__ __forceinline__ void table_locate(const TabMeta<T>& tm, T x, int& idx, T& xx, T& delta) {
  xx = x;
  delta = (T)0;
  if (xx < tm.lower) {
    idx = 0;
    delta = xx - tm.lower;
    xx = (T)0;
  } else if (xx < tm.upper) {
    idx = (int)((xx - tm.lower) / tm.s0);
    xx -= (idx * tm.s0 + tm.lower);
  } else if (xx < tm.mx) {
    idx = tm.first + (int)((xx - tm.upper) / tm.s1);
    xx -= ((idx - tm.first) * tm.s1 + tm.upper);
  } else {
    idx = tm.hi_idx;
    delta = xx - tm.mx;
    xx = tm.hi_xx;
  }
}

// Embedding nets: all nets share widths; W[l] is [nnets, nin_l, nout_l],
// b[l] / idt[l] are [nnets, nout_l] (idt NULL when the layer has none).
template <typename T>
struct EmbParams {
  int n_layer;
  int width[kMaxEmbLayers];  // output widths; input of layer 0 is 1
  const T* W[kMaxEmbLayers];
  const T* b[kMaxEmbLayers];
  const T* idt[kMaxEmbLayers];
  int compressed;
  const T* table;            // compressed: all nets' tables
  const TabMeta<T>* meta;    // compressed: [nnets]
};

template <typename T>
struct DescParams {
  int nloc;       // atoms per frame
  int nrows;      // nframes * nloc
  int nnei;
  int ntypes;
  int sec[DPGB_MAX_TYPES + 1];
  int type_one_side;
  int ng, axis;
  int pad_zero;   // padding slots contribute exactly zero (mean == 0)
  double rcut, rcut_smth;
  const T* davg;  // [ntypes, nnei, 4]
  const T* dstd;
  const T* dstd_inv;  // 1 / dstd (the mixed-precision kernels multiply)
  FastDiv nloc_div;   // division by nloc
  const int* pair_mask;     // [ntypes*ntypes] or NULL
  const double* coord;      // [nframes, nloc, 3] normalised
  const int* atype;         // [nloc]
  const int* nlist;         // [nrows, nnei] extended indices (image-major)
  const double* svec;       // [nframes, nshift, 3] image shift vectors
  int nshift;
  const int* row_pos;       // [nrows] sorted (by type) row of each atom
  // explicit extended atoms (an external neighbour list with ghost atoms,
  // as LAMMPS passes them): when coord_ext is set, nlist holds indices into
  // coord_ext [nframes, nall, 3] / atype_ext [nframes, nall] (local atoms
  // first) instead of image-major extended indices
  const double* coord_ext;
  const int* atype_ext;
  int nall;
  // a batch of frames of different sizes run as one "frame" of all their
  // atoms: when frame_atom_off is set, row r belongs to the frame f with
  // frame_atom_off[f] <= r < frame_atom_off[f+1], nlist holds that frame's
  // image-major indices and its shifts start at svec[3 * frame_svec_off[f]]
  const int* frame_atom_off;
  const int* frame_svec_off;
  int nframes_batch;
  // FP32 split (x = hi + lo) of the coordinates ([nrows], or [nframes, nall]
  // with coord_ext) and of the shift vectors (as svec), for FP32
  // displacements (pair_disp_f); NULL: displacements in FP64
  const float4* xhi;
  const float4* xlo;
  const float4* shi;
  const float4* slo;
  // forces as 2^-32 fixed-point integers [nrows][3] (model lists): when set,
  // the table backward adds each pair's gradient onto its row and its
  // neighbour's row with 64-bit integer atomics instead of storing it
  unsigned long long* facc;
};

// The row whose force takes the neighbour's share of pair (row, nb): the
// explicit extended atom nb with an external list (ghosts included), else
// atom nb mod (the frame's atom count) of the row's frame (image-major index
// nb; a batch's frames are found from frame_atom_off).
// KEY: the list kind when known at compile time (kKeyModel, kKeyBatch,
// kKeyExt), or kKeyAny to decide from p.
enum { kKeyModel = 0, kKeyBatch = 1, kKeyExt = 2, kKeyAny = 3 };
template <int KEY = kKeyAny, typename T>
__device__ __forceinline__ int neighbour_row(const DescParams<T>& p, int row, int nb) {
  if (KEY == kKeyExt || (KEY == kKeyAny && p.coord_ext)) return nb;
  if (KEY == kKeyBatch || (KEY == kKeyAny && p.frame_atom_off)) {
    const int f = frame_of(p.frame_atom_off, p.nframes_batch, row);
    const int beg = p.frame_atom_off[f];
    return beg + nb % (p.frame_atom_off[f + 1] - beg);
  }
  return p.nloc_div.div(row) * p.nloc + nb - p.nloc_div.div(nb) * p.nloc;
}
template <typename T>
__host__ __device__ inline int list_key_kind(const DescParams<T>& p) {
  return p.coord_ext ? kKeyExt : (p.frame_atom_off ? kKeyBatch : kKeyModel);
}

// r_nb - r_i in FP64 for neighbour nb of local atom i of frame f, and the
// neighbour's type.  Image-major indices: r_nb = coord[nb % nloc] + shift.
template <typename T>
__device__ __forceinline__ int pair_disp(const DescParams<T>& p, int f, int i, int nb, double d[3]) {
  if (p.coord_ext) {
    const double* ce = p.coord_ext + (size_t)f * p.nall * 3;
    d[0] = ce[3 * nb] - ce[3 * i];
    d[1] = ce[3 * nb + 1] - ce[3 * i + 1];
    d[2] = ce[3 * nb + 2] - ce[3 * i + 2];
    return p.atype_ext[(size_t)f * p.nall + nb];
  }
  if (p.frame_atom_off) {  // batch: i is the global row
    const int fr = frame_of(p.frame_atom_off, p.nframes_batch, i);
    const int beg = p.frame_atom_off[fr], nl = p.frame_atom_off[fr + 1] - beg;
    const int s = nb / nl, jj = beg + (nb - s * nl);
    const double* sv = p.svec + 3 * ((size_t)p.frame_svec_off[fr] + s);
    d[0] = (p.coord[3 * jj] + sv[0]) - p.coord[3 * i];
    d[1] = (p.coord[3 * jj + 1] + sv[1]) - p.coord[3 * i + 1];
    d[2] = (p.coord[3 * jj + 2] + sv[2]) - p.coord[3 * i + 2];
    return p.atype[jj];
  }
  const double* cf = p.coord + (size_t)f * p.nloc * 3;
  const int s = nb / p.nloc, jj = nb - s * p.nloc;
  const double* sv = p.svec + ((size_t)f * p.nshift + s) * 3;
  d[0] = (cf[3 * jj] + sv[0]) - cf[3 * i];
  d[1] = (cf[3 * jj + 1] + sv[1]) - cf[3 * i + 1];
  d[2] = (cf[3 * jj + 2] + sv[2]) - cf[3 * i + 2];
  return p.atype[jj];
}

// pair_disp rounded to FP32: from the FP32 splits when the params carry
// them, else from the FP64 displacement
template <typename T>
__device__ __forceinline__ int pair_disp_f(const DescParams<T>& p, int f, int i, int nb, float d[3]) {
  if (!p.xhi) {
    double dd[3];
    const int t = pair_disp(p, f, i, nb, dd);
    d[0] = (float)dd[0];
    d[1] = (float)dd[1];
    d[2] = (float)dd[2];
    return t;
  }
  size_t aj, ai, sv = 0;
  bool shift = true;
  int t;
  if (p.coord_ext) {
    aj = (size_t)f * p.nall + nb;
    ai = (size_t)f * p.nall + i;
    shift = false;
    t = p.atype_ext[aj];
  } else if (p.frame_atom_off) {
    const int fr = frame_of(p.frame_atom_off, p.nframes_batch, i);
    const int beg = p.frame_atom_off[fr], nl = p.frame_atom_off[fr + 1] - beg;
    const int s = nb / nl, jj = beg + (nb - s * nl);
    aj = jj;
    ai = i;
    sv = (size_t)p.frame_svec_off[fr] + s;
    t = p.atype[jj];
  } else {
    const int s = p.nloc_div.div(nb), jj = nb - s * p.nloc;
    aj = (size_t)f * p.nloc + jj;
    ai = (size_t)f * p.nloc + i;
    sv = (size_t)f * p.nshift + s;
    t = p.atype[jj];
  }
  const float4 jh = p.xhi[aj], jl = p.xlo[aj], ih = p.xhi[ai], il = p.xlo[ai];
  const float4 sh = shift ? p.shi[sv] : make_float4(0.f, 0.f, 0.f, 0.f);
  const float4 sl = shift ? p.slo[sv] : make_float4(0.f, 0.f, 0.f, 0.f);
  d[0] = disp_split(jh.x, jl.x, sh.x, sl.x, ih.x, il.x);
  d[1] = disp_split(jh.y, jl.y, sh.y, sl.y, ih.y, il.y);
  d[2] = disp_split(jh.z, jl.z, sh.z, sl.z, ih.z, il.z);
  return t;
}

// Fitting nets of all types: W[l] [ntypes, nin_l, nout_l] ...
template <typename T>
struct FitParams {
  int n_hidden;
  int width[kMaxFitLayers + 1];  // width[0] = dim_descrpt, width[l+1] = hidden l
  const T* W[kMaxFitLayers];
  const T* b[kMaxFitLayers];
  const T* idt[kMaxFitLayers];
  const T* w_out;  // [ntypes, width[n_hidden]]
  const T* b_out;  // [ntypes]
};

// Buffers of one evaluation (rows in type-sorted order unless stated).
template <typename T>
struct Work {
  T* D;      // [nrows, dim]
  T* dD;     // [nrows, dim]
  T* xyz;    // [nrows, 4, ng] original row order
  T* gpair;  // [nrows, nnei, 3] original row order
  double* vir_row;   // [nrows, 9]
  double* e_row;     // [nrows] atom energy, original order
  T* act;    // fitting activations: per hidden layer Y and tanh T: 2*n_hidden*[nrows, maxw]
  T* gbuf;   // fitting gradients: 2 * [nrows, maxw]
};

template <typename T>
int launch_desc_fwd(const DescParams<T>& p, const EmbParams<T>& e, T* D, T* xyz, size_t smem,
                    cudaStream_t st);
template <typename T>
size_t desc_fwd_smem(const DescParams<T>& p, const EmbParams<T>& e);
template <typename T>
int launch_desc_bwd(const DescParams<T>& p, const EmbParams<T>& e, const T* dD, const T* xyz,
                    T* gpair, double* vir_row, size_t smem, cudaStream_t st);
template <typename T>
size_t desc_bwd_smem(const DescParams<T>& p, const EmbParams<T>& e);

// Compressed nets in the mixed form (tab_fused.cu): the table lookup fused
// with the env matrix and contraction (forward: xyz in row order, D at the
// type-sorted position, BF16 when d_bf16) and the pair-gradient backward.
// Work: the chunks of type-sorted rows (one centre type each); D is
// written at the type-sorted position.
struct WorkChunk;
int tab_fused_eligible(int ng, int axis);
// env_out / env_in: [nrows][nnei][2] float4 (R~; displacement, kept flag)
// of the real pairs, written by the forward and read by the backward (NULL:
// the backward forms the environment itself)
int launch_tab_fwd(const DescParams<float>& p, const EmbParams<float>& e, const WorkChunk* chunks, int nchunks,
                   const int* sorted_rows, float* xyz, void* D, int d_bf16, cudaStream_t st, int* queue = nullptr,
                   float4* env_out = nullptr);
int launch_tab_bwd(const DescParams<float>& p, const EmbParams<float>& e, const WorkChunk* chunks, int nchunks,
                   const int* sorted_rows, const float* dxyz, float* gpair, double* vir_row, cudaStream_t st,
                   int* queue = nullptr, const float4* env_in = nullptr);

// fitting of the rows [row0, row0+nrow) of one type
template <typename T>
int launch_fitting(const FitParams<T>& f, int type, int row0, int nrow, int nrows_total,
                   const T* D, T* dD, T* act, T* gbuf, double* e_sorted, double ener_bias,
                   cudaStream_t st);

}  // namespace dpgb
