// Tensor-core (tcgen05) form of the se_e2_a embedding for the mixed-precision
// DeepPot: forward (G, xyz, D) and backward (pair gradients, virial).
#pragma once

#include "se_a.cuh"

namespace dpgb {

constexpr int kTcRows = 128;     // MMA M: pairs per tile
constexpr int kTcMaxAtoms = 16;  // atoms per tile

// Column order of a layer's outputs (its TMEM accumulator columns, and the K
// order of the next layer's operand).  When the layer doubles its input
// through the residual (w_out == 2 w_in: the skip adds the input to both
// halves), each group of 16 columns holds 8 consecutive neurons m of the
// first half and their partners w_in + m, so the two contributions to one
// input neuron meet in one group (the backward folds them group by group).
// Otherwise the natural order.  -1: a padding column.  The padded width
// 16 * ceil(w_in / 8) equals pad16(w_out).
__host__ __device__ constexpr int col_neuron(int c, int w_out, int w_in) {
  return w_out != 2 * w_in ? (c < w_out ? c : -1)
                           : ((8 * (c >> 4) + (c & 7)) >= w_in ? -1
                                                               : ((c & 15) < 8 ? 8 * (c >> 4) + (c & 7)
                                                                               : w_in + 8 * (c >> 4) + (c & 7)));
}
__host__ __device__ constexpr int neuron_col(int n, int w_out, int w_in) {
  return w_out != 2 * w_in ? n
                           : 16 * ((n < w_in ? n : n - w_in) >> 3) + (n < w_in ? 0 : 8) + ((n < w_in ? n : n - w_in) & 7);
}

// The k-th padding column (k = 0, 1) of a layer's n padded output columns.
// The next layer's bias rides in the MMA on two such columns: the operand
// holds 1 there and the weight image the bias split into BF16 hi + lo, so
// the accumulator arrives with the bias added (to ~2^-17 of it).  The first
// layer's outputs use their natural order: columns w1 and w1 + 1.
__host__ __device__ constexpr int bias_col(int k, int w_out, int w_in, int n) {
  for (int c = 0; c < n; ++c)
    if (col_neuron(c, w_out, w_in) < 0 && k-- == 0) return c;
  return -1;
}

// Per-net weight images (bf16, already in the shared-memory core-matrix
// layout) and FP32 vectors of a 3-layer embedding net 1 -> w1 -> w2 -> w3.
// Layer-2 and layer-3 outputs are in col_neuron order (rows of fw2 / fw3,
// K of fw3 / bw2 / bw3, the b/idt vectors of layers 2 and 3).
struct EmbTC {
  int w1, w2, w3;        // real widths
  int k1, n2, n3;        // padded: k1 = pad16(w1), n2 = pad16(w2), n3 = pad16(w3)
  int nnets;
  // [nnets][...] images, byte sizes per net below
  const unsigned char* fw2;  // forward B of layer 2: W2^T [n2 x k1]
  const unsigned char* fw3;  // forward B of layer 3: W3^T [n3 x n2]
  const unsigned char* bw3;  // backward B of layer 3: W3 [n2 x n3]
  const unsigned char* bw2;  // backward B of layer 2: W2 [k1 x n2]
  const unsigned char* fw2lo;  // low BF16 parts of fw2 (the forward's weights are split BF16)
  const unsigned char* fw3lo;  // low BF16 parts of fw3
  const float* vec;          // [nnets][vec_stride]: w1 b1 idt1 | b2 idt2 | b3 idt3 (padded; b2, b3 also ride
                             // in fw2 / fw3 on the bias columns, which is where the kernels take them from)
  int vec_stride;
  int has_idt1, has_idt2, has_idt3;
  int d_bf16;  // per call: write D as BF16 (for the tensor-core fitting)
};

// contiguous ranges of type-sorted rows processed by one CTA (same centre
// type): the work items of the persistent embedding and table kernels
struct WorkChunk {
  int row0, row1;  // sorted-row range [row0, row1)
  int ti;          // centre type
  int pad;
};

template <typename T>
struct DescParams;

int emb_tc_eligible(const dpgb_se_a_desc& d);
int build_emb_tc(const dpgb_se_a_desc& d, std::vector<unsigned char>& images, EmbTC& meta,
                 std::vector<float>& vec);
// fill device pointers of meta from one device buffer holding images then vec
void emb_tc_bind(EmbTC& meta, const unsigned char* dev_images, size_t img_bytes_per_kind, const float* dev_vec);
size_t emb_tc_image_bytes(const EmbTC& m, int kind);  // per net: 0 fw2, 1 fw3, 2 bw3, 3 bw2, 4 fw2lo, 5 fw3lo

// queue: NULL = the work items go to the CTAs in a fixed stride; else an
// int the caller zeroed on the stream, from which the CTAs draw the items
int launch_run_lengths(int* run_len, const int* nlist, const int* sorted_rows, int nrows, int nnei,
                       const SelInfo& sel, int pad_zero, cudaStream_t st);
// xyzp: per-section partial xyz by accumulator column, [ntypes][nrows][4][pad16(ng)] FP32 scratch
int launch_emb_tc_fwd(const DescParams<float>& p, const EmbTC& e, const WorkChunk* chunks, int nchunks,
                      const int* run_len, const int* sorted_rows, float* xyz, float* xyzp, float* D, int* status,
                      cudaStream_t st, int* queue = nullptr);
int launch_dxyz(const DescParams<float>& p, const float* dD, const float* xyz, float* dxyz, cudaStream_t st);
int launch_emb_tc_bwd(const DescParams<float>& p, const EmbTC& e, const WorkChunk* chunks, int nchunks,
                      const int* run_len, const int* sorted_rows, const float* dxyz, float* gpair,
                      double* vir_row, int* status, cudaStream_t st, int* queue = nullptr);

}  // namespace dpgb
