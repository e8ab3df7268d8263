// Tensor-core (tcgen05) form of the se_e2_a embedding for the mixed-precision
// DeepPot: forward (G, xyz, D) and backward (pair gradients, virial).
#pragma once

#include "se_a.cuh"

namespace dpgb {

constexpr int kTcRows = 128;     // MMA M: pairs per tile
constexpr int kTcMaxAtoms = 16;  // atoms per tile

// Per-net weight images (bf16, already in the shared-memory core-matrix
// layout) and FP32 vectors of a 3-layer embedding net 1 -> w1 -> w2 -> w3.
struct EmbTC {
  int w1, w2, w3;        // real widths
  int k1, n2, n3;        // padded: k1 = pad16(w1), n2 = pad16(w2), n3 = pad16(w3)
  int nnets;
  // [nnets][...] images, byte sizes per net below
  const unsigned char* fw2;  // forward B of layer 2: W2^T [n2 x k1]
  const unsigned char* fw3;  // forward B of layer 3: W3^T [n3 x n2]
  const unsigned char* bw3;  // backward B of layer 3: W3 [n2 x n3]
  const unsigned char* bw2;  // backward B of layer 2: W2 [k1 x n2]
  const float* vec;          // [nnets][vec_stride]: w1 b1 idt1 | b2 idt2 | b3 idt3 (padded)
  int vec_stride;
  int has_idt1, has_idt2, has_idt3;
  int d_bf16;  // per call: write D as BF16 (for the tensor-core fitting)
};

// contiguous ranges of type-sorted rows processed by one CTA (same centre type)
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
size_t emb_tc_image_bytes(const EmbTC& m, int kind);  // per net: 0 fw2, 1 fw3, 2 bw3, 3 bw2

int launch_run_lengths(int* run_len, const int* nlist, const int* sorted_rows, int nrows, int nnei,
                       const SelInfo& sel, int pad_zero, cudaStream_t st);
// xyzp: per-section partial xyz, [ntypes][nrows][4][ng] FP32 scratch
int launch_emb_tc_fwd(const DescParams<float>& p, const EmbTC& e, const WorkChunk* chunks, int nchunks,
                      const int* run_len, const int* sorted_rows, float* xyz, float* xyzp, float* D, int* status,
                      cudaStream_t st);
int launch_dxyz(const DescParams<float>& p, const float* dD, const float* xyz, float* dxyz, cudaStream_t st);
int launch_emb_tc_bwd(const DescParams<float>& p, const EmbTC& e, const WorkChunk* chunks, int nchunks,
                      const int* run_len, const int* sorted_rows, const float* dxyz, float* gpair,
                      double* vir_row, int* status, cudaStream_t st);

}  // namespace dpgb
