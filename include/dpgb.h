/* dpgb — GB300-native (sm_103a) se_e2_a energy / force / virial library.
 *
 * Plain C ABI: device or host pointers and sizes, no C++ or torch types.
 * Every function returns 0 on success or a negative DPGB_E* code; the text of
 * the last error of the calling thread is returned by dpgb_last_error().
 * Kernels are enqueued on the caller's stream (`stream` is a cudaStream_t,
 * NULL = the legacy default stream); functions that return device results do
 * not synchronise unless they say so.  No function uses atomics for floating
 * point accumulation: results are bitwise reproducible run to run.
 *
 * Each declaration names the reference interface it replaces (paths in the
 * deepmodeling/deepmd-kit tree).
 */
#ifndef DPGB_H
#define DPGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DPGB_OK 0
#define DPGB_EINVAL -1    /* bad argument (sizes, NULL pointers, dims) */
#define DPGB_ECUDA -2     /* a CUDA runtime call failed */
#define DPGB_EOVERFLOW -3 /* a neighbour buffer or bucket capacity was exceeded */
#define DPGB_ENOMEM -4    /* device allocation failed */
#define DPGB_ETIMEOUT -5  /* a bounded device-side wait gave up */

#define DPGB_MAX_TYPES 8
#define DPGB_MAX_LAYERS 6

/* Text of the last error raised on the calling thread ("" when none). */
const char* dpgb_last_error(void);
/* Library version string. */
const char* dpgb_version(void);

/* ------------------------------------------------------------------------
 * tabulate_fusion_se_a — the compressed embedding fused with G^T R~.
 * Replaces deepmd::tabulate_fusion_se_a_gpu / _grad_gpu / _grad_grad_gpu
 * (source/lib/include/tabulate.h:11-71, source/lib/src/gpu/tabulate.cu:
 * 1218-1367) behind torch.ops.deepmd.tabulate_fusion_se_a
 * (source/op/pt/tabulate_multi_device.cc:1630).  Device pointers:
 *   table [nspline, 6*last_layer_size], em_x [nloc*nnei], em [nloc,nnei,4],
 *   out / dz_dy [nloc, 4, last_layer_size], dy [nloc, 4, last_layer_size],
 *   dy_dem_x [nloc*nnei], dy_dem [nloc, nnei, 4].
 * table_info is a HOST array of 6: {lower, upper, upper*extrapolate,
 * stride0, stride1, check_frequency} (tabulate_multi_device.cc:33-49).
 * is_sorted folds trailing padding exactly like the reference. */
int dpgb_tabulate_fusion_se_a_f64(double* out, const double* table,
                                  const double* table_info_host,
                                  const double* em_x, const double* em,
                                  int nloc, int nnei, int last_layer_size,
                                  int is_sorted, void* stream);
int dpgb_tabulate_fusion_se_a_f32(float* out, const float* table,
                                  const float* table_info_host,
                                  const float* em_x, const float* em, int nloc,
                                  int nnei, int last_layer_size, int is_sorted,
                                  void* stream);
int dpgb_tabulate_fusion_se_a_grad_f64(double* dy_dem_x, double* dy_dem,
                                       const double* table,
                                       const double* table_info_host,
                                       const double* em_x, const double* em,
                                       const double* dy, int nloc, int nnei,
                                       int last_layer_size, int is_sorted,
                                       void* stream);
int dpgb_tabulate_fusion_se_a_grad_f32(float* dy_dem_x, float* dy_dem,
                                       const float* table,
                                       const float* table_info_host,
                                       const float* em_x, const float* em,
                                       const float* dy, int nloc, int nnei,
                                       int last_layer_size, int is_sorted,
                                       void* stream);
int dpgb_tabulate_fusion_se_a_grad_grad_f64(
    double* dz_dy, const double* table, const double* table_info_host,
    const double* em_x, const double* em, const double* dz_dy_dem_x,
    const double* dz_dy_dem, int nloc, int nnei, int last_layer_size,
    int is_sorted, void* stream);
int dpgb_tabulate_fusion_se_a_grad_grad_f32(
    float* dz_dy, const float* table, const float* table_info_host,
    const float* em_x, const float* em, const float* dz_dy_dem_x,
    const float* dz_dy_dem, int nloc, int nnei, int last_layer_size,
    int is_sorted, void* stream);

/* ------------------------------------------------------------------------
 * Neighbour lists.
 *
 * dpgb_format_nlist_a: format a candidate list into typed sections.
 * Replaces deepmd::format_nbor_list_gpu (source/lib/src/gpu/
 * prod_env_mat.cu:618-679) / format_nlist_cpu (source/lib/src/fmt_nlist.cc:
 * 98-150).  Candidates come as a dense device array in_rows [nloc, max_nbor]
 * with in_counts [nloc] (the reference's InputNlist ilist/numneigh/
 * firstneigh, ilist = identity).  Order: (type, fp32 r^2, index), each type
 * truncated to sel[t]; nlist [nloc, sum(sel)] (-1 padded).  *overflow_host
 * (optional) receives the number of rows that dropped neighbours; passing it
 * synchronises the stream.  Returns DPGB_EOVERFLOW when a row holds more than
 * 1024 candidates within rcut. */
int dpgb_format_nlist_a(int* nlist, const double* coord_ext, const int* atype_ext,
                        const int* in_rows, const int* in_counts, int max_nbor,
                        int nloc, int nall, double rcut, const int* sel_host,
                        int ntypes, int* overflow_host, void* stream);

/* dpgb_build_nlist_pt: typed neighbour list of one periodic (or open) frame
 * in the order of the reference PyTorch path: extended atoms (all periodic
 * images, image-major, images in the order `shift_idx` gives) within rcut
 * ordered by (fp64 distance, extended index), the nearest sum(sel) kept, then
 * split per type keeping the first sel[t] (deepmd/pt/utils/nlist.py:14-199,
 * 304-337, 424-513).  Built with a cell list in O(N).
 *   coord [nloc,3] (already normalised), atype [nloc] (device),
 *   box_host [9] (NULL = open boundary), shift_idx_host [nshift, 3] integer
 *   image shifts in reference order (ignored when box_host is NULL),
 *   nlist [nloc, sum(sel)] extended indices, -1 padded (device).
 * Returns DPGB_EOVERFLOW when an atom has more than 1024 atoms within rcut. */
int dpgb_build_nlist_pt(int* nlist, const double* coord, const int* atype,
                        int nloc, const double* box_host,
                        const int* shift_idx_host, int nshift, double rcut,
                        const int* sel_host, int ntypes, void* stream);

/* The three steps above for nframes periodic frames at once, as
 * extend_input_and_build_neighbor_list (deepmd/pt/utils/nlist.py:14-46)
 * does for a batch: every frame wrapped (normalize_coord), its images in the
 * order shift_idx gives (one table for all frames: the reference takes the
 * largest image count over the batch) and its typed list; one workspace,
 * one status read (synchronises the stream once).
 *   coord [nframes, nloc, 3], atype [nframes, nloc] (device), box_host
 *   [nframes, 9] -> coord_ext [nframes, nshift * nloc, 3], atype_ext,
 *   mapping [nframes, nshift * nloc], nlist [nframes, nloc, sum(sel)]
 *   (device).  Non-finite coordinates or cells return DPGB_EINVAL. */
int dpgb_extend_input_and_build_nlist(double* coord_ext, int* atype_ext,
                                      int* mapping, int* nlist,
                                      const double* coord, const int* atype,
                                      int nframes, int nloc,
                                      const double* box_host,
                                      const int* shift_idx_host, int nshift,
                                      double rcut, const int* sel_host,
                                      int ntypes, void* stream);

/* Periodic wrap of coordinates into the cell: deepmd/pt/utils/region.py:86
 * normalize_coord / source/lib/src/gpu/coord.cu:45 normalize_one. */
int dpgb_normalize_coord(double* coord_out, const double* coord, int natom,
                         const double* box_host, void* stream);

/* Extended (ghost) coordinates, types and mapping in the reference PyTorch
 * layout: ext[s*nloc + j] = coord[j] + shift_idx[s] . box
 * (deepmd/pt/utils/nlist.py:424-513).  Device outputs sized nshift*nloc. */
int dpgb_extend_coord(double* coord_ext, int* atype_ext, int* mapping,
                      const double* coord, const int* atype, int nloc,
                      const double* box_host, const int* shift_idx_host,
                      int nshift, void* stream);

/* ------------------------------------------------------------------------
 * Environment matrix.  Replaces deepmd::prod_env_mat_a_gpu
 * (source/lib/include/prod_env_mat.h, source/lib/src/gpu/prod_env_mat.cu:
 * 681-726): formats the candidate list (dpgb_format_nlist_a) and evaluates
 * em [nloc, nnei, 4] = (R~ - avg[t_i]) / std[t_i],
 * em_deriv [nloc, nnei, 4, 3] = dR~/d r_centre / std, rij [nloc, nnei, 3],
 * nlist [nloc, nnei].  avg/std [ntypes, nnei, 4] device. */
int dpgb_prod_env_mat_a_f64(double* em, double* em_deriv, double* rij,
                            int* nlist, const double* coord_ext,
                            const int* atype_ext, const int* in_rows,
                            const int* in_counts, int max_nbor,
                            const double* avg, const double* std, int nloc,
                            int nall, double rcut, double rcut_smth,
                            const int* sel_host, int ntypes, void* stream);

/* Environment matrix of an already typed list, PyTorch API semantics
 * (deepmd/pt/model/descriptor/env_mat.py:18-119 prod_env_mat): every
 * non-negative slot evaluated, padding = (0 - avg)/std.  Outputs em
 * [nf*nloc, nnei, 4], diff [.., 3], sw [.., 1]; nlist holds extended indices
 * into coord_ext [nf, nall, 3]. */
int dpgb_env_mat_pt_f64(double* em, double* diff, double* sw,
                        const double* coord_ext, const int* atype_ext,
                        const int* nlist, const double* avg, const double* std,
                        int nf, int nloc, int nall, int nnei, double rcut,
                        double rcut_smth, void* stream);

/* The same with the reference's `protection` (added to the distance in the
 * 1/r and 1/r^2 factors, env_mat.py:41-43), in FP32 or FP64 (the
 * descriptor's `precision`), and with the local types atype [nf, nloc] of
 * the reference signature (env_mat.py:58-70) instead of atype_ext. */
int dpgb_env_mat_pt2_f64(double* em, double* diff, double* sw,
                         const double* coord_ext, const int* atype,
                         const int* nlist, const double* avg, const double* std,
                         int nf, int nloc, int nall, int nnei, double rcut,
                         double rcut_smth, double protection, void* stream);
int dpgb_env_mat_pt2_f32(float* em, float* diff, float* sw,
                         const float* coord_ext, const int* atype,
                         const int* nlist, const float* avg, const float* std,
                         int nf, int nloc, int nall, int nnei, double rcut,
                         double rcut_smth, double protection, void* stream);

/* Backward of prod_env_mat with respect to the extended coordinates: the
 * gradient autograd forms through env_mat.py:18-119.  g_em [nf*nloc, nnei, 4],
 * g_diff [.., 3] and g_sw [.., 1] (either may be NULL) -> g_coord
 * [nf, nall, 3] (overwritten).  Pair terms are gathered per atom through a
 * sorted transpose of the list: no atomics, reproducible. */
int dpgb_env_mat_pt_bwd_f64(double* g_coord, const double* g_em,
                            const double* g_diff, const double* g_sw,
                            const double* coord_ext, const int* atype,
                            const int* nlist, const double* std, int nf,
                            int nloc, int nall, int nnei, double rcut,
                            double rcut_smth, double protection, void* stream);
int dpgb_env_mat_pt_bwd_f32(float* g_coord, const float* g_em,
                            const float* g_diff, const float* g_sw,
                            const float* coord_ext, const int* atype,
                            const int* nlist, const float* std, int nf,
                            int nloc, int nall, int nnei, double rcut,
                            double rcut_smth, double protection, void* stream);

/* Second derivative: the backward of dpgb_env_mat_pt_bwd.  Given the
 * cotangent u [nf, nall, 3] of g_coord: gg_em [nf*nloc, nnei, 4] and
 * gg_diff / gg_sw (either may be NULL) receive the directional derivatives
 * of em / diff / sw along u (the map is linear in g_em, g_diff, g_sw), and
 * gg_coord [nf, nall, 3] (may be NULL) the curvature term
 * sum g . (d2 em / dr2) u. */
int dpgb_env_mat_pt_bwd_bwd_f64(double* gg_em, double* gg_diff, double* gg_sw,
                                double* gg_coord, const double* u,
                                const double* g_em, const double* g_diff,
                                const double* g_sw, const double* coord_ext,
                                const int* atype, const int* nlist,
                                const double* std, int nf, int nloc, int nall,
                                int nnei, double rcut, double rcut_smth,
                                double protection, void* stream);
int dpgb_env_mat_pt_bwd_bwd_f32(float* gg_em, float* gg_diff, float* gg_sw,
                                float* gg_coord, const float* u,
                                const float* g_em, const float* g_diff,
                                const float* g_sw, const float* coord_ext,
                                const int* atype, const int* nlist,
                                const float* std, int nf, int nloc, int nall,
                                int nnei, double rcut, double rcut_smth,
                                double protection, void* stream);

/* ------------------------------------------------------------------------
 * se_e2_a descriptor block on an environment matrix, with first and second
 * derivatives: the operator behind DescrptBlockSeA.forward
 * (deepmd/pt/model/descriptor/se_a.py:742-858).  The embedding nets'
 * parameters are one flat device vector: for each net e (e = ii for
 * type_one_side, else e = ii * ntypes + ti, ii the neighbour type and ti the
 * centre type, se_a.py:805-808) and each layer l: matrix [nin_l, nout_l]
 * row-major, bias [nout_l], then idt [nout_l] when resnet_dt.
 * pair_keep is the (ntypes+1)^2 exclusion table of PairExcludeMask
 * (deepmd/pt/utils/exclude_mask.py:64-141; the last type is the padding),
 * laid out with a row stride of DPGB_MAX_TYPES + 1; 1 keeps a pair. */
typedef struct dpgb_se_a_block {
  int ntypes;
  int sel[DPGB_MAX_TYPES];
  int type_one_side;
  int n_layer;
  int neuron[DPGB_MAX_LAYERS];
  int axis_neuron;
  int resnet_dt;
  int pair_keep[(DPGB_MAX_TYPES + 1) * (DPGB_MAX_TYPES + 1)];
} dpgb_se_a_block;

/* Compression table of one embedding net, built on the device: replaces
 * DPTabulate._build_lower / _make_data (deepmd/utils/tabulate.py:275-370,
 * deepmd/utils/tabulate_math.py:353-470) for se_e2_a.  params is the flat
 * parameter vector described below, `net` the net index.  table
 * [nrows, 6 * ng] (device) with nrows = dpgb_se_a_table_rows(...), the
 * reference's int((upper - lower)/stride0 + (extrapolate*upper - upper)/
 * stride1).  Synchronises the stream. */
int dpgb_se_a_table_rows(double lower, double upper, double extrapolate,
                         double stride0, double stride1);
struct dpgb_se_a_block;
int dpgb_se_a_table_build_f64(double* table, const struct dpgb_se_a_block* b,
                              const double* params, int net, double lower,
                              double upper, double extrapolate, double stride0,
                              double stride1, void* stream);

/* Number of parameters in the flat vector (-1 for a bad description). */
long long dpgb_se_a_block_param_count(const dpgb_se_a_block* b);
/* Workspace the parameter gradient needs (bytes) for nf * nloc rows at
 * precision_bytes (8 or 4) per element. */
size_t dpgb_se_a_block_workspace_bytes(const dpgb_se_a_block* b, int nf,
                                       int nloc, int precision_bytes);

/* Forward: rr [nf*nloc, nnei, 4] (normalised env matrix), nlist
 * [nf*nloc, nnei], atype_ext [nf, nall] -> descriptor [nf*nloc, ng*M] and
 * xyz [nf*nloc, 4, ng] (the reference's xyz_scatter / nnei; rot_mat is
 * xyz^T[:, 1:4]). */
int dpgb_se_a_block_fwd_f64(const dpgb_se_a_block* b, const double* params,
                            const double* rr, const int* nlist,
                            const int* atype_ext, int nf, int nloc, int nall,
                            double* descriptor, double* xyz, void* stream);
int dpgb_se_a_block_fwd_f32(const dpgb_se_a_block* b, const float* params,
                            const float* rr, const int* nlist,
                            const int* atype_ext, int nf, int nloc, int nall,
                            float* descriptor, float* xyz, void* stream);

/* Backward: cotangents of descriptor and (optionally) xyz -> g_rr
 * [nf*nloc, nnei, 4] and, when g_params is not NULL, the parameter gradient
 * (needs the workspace).  xyz is the forward's output. */
int dpgb_se_a_block_bwd_f64(const dpgb_se_a_block* b, const double* params,
                            const double* rr, const int* nlist,
                            const int* atype_ext, int nf, int nloc, int nall,
                            const double* xyz, const double* g_descriptor,
                            const double* g_xyz, double* g_rr,
                            double* g_params, void* workspace,
                            size_t workspace_bytes, void* stream);
int dpgb_se_a_block_bwd_f32(const dpgb_se_a_block* b, const float* params,
                            const float* rr, const int* nlist,
                            const int* atype_ext, int nf, int nloc, int nall,
                            const float* xyz, const float* g_descriptor,
                            const float* g_xyz, float* g_rr, float* g_params,
                            void* workspace, size_t workspace_bytes,
                            void* stream);

/* Double backward: the backward of the backward, for the cotangent u_rr of
 * g_rr (training on forces).  Outputs the cotangents of g_descriptor
 * (gg_descriptor), of g_xyz (gg_xyz, may be NULL), of rr (gg_rr) and of the
 * parameters (gg_params, may be NULL; needs the workspace).  Activations are
 * recomputed, never stored. */
int dpgb_se_a_block_bwd_bwd_f64(const dpgb_se_a_block* b, const double* params,
                                const double* rr, const int* nlist,
                                const int* atype_ext, int nf, int nloc,
                                int nall, const double* g_descriptor,
                                const double* g_xyz, const double* u_rr,
                                double* gg_descriptor, double* gg_xyz,
                                double* gg_rr, double* gg_params,
                                void* workspace, size_t workspace_bytes,
                                void* stream);
int dpgb_se_a_block_bwd_bwd_f32(const dpgb_se_a_block* b, const float* params,
                                const float* rr, const int* nlist,
                                const int* atype_ext, int nf, int nloc,
                                int nall, const float* g_descriptor,
                                const float* g_xyz, const float* u_rr,
                                float* gg_descriptor, float* gg_xyz,
                                float* gg_rr, float* gg_params,
                                void* workspace, size_t workspace_bytes,
                                void* stream);

/* ------------------------------------------------------------------------
 * Force and virial from net_deriv = dE/d em.  Replace deepmd::prod_force_a_gpu
 * (source/lib/src/gpu/prod_force.cu:4-130) and prod_virial_a_gpu
 * (prod_virial.cu:4-134) without atomics: neighbour contributions are
 * gathered through a sorted transpose of the list.
 *   net_deriv [nf*nloc, 4*nnei], env_deriv [nf*nloc, 4*nnei, 3],
 *   rij [nloc, nnei, 3], nlist [nf*nloc, nnei] (indices < nall),
 *   force [nf, nall, 3], virial [9], atom_virial [nall, 9]. */
int dpgb_prod_force_a_f64(double* force, const double* net_deriv,
                          const double* env_deriv, const int* nlist, int nloc,
                          int nall, int nnei, int nframes, void* stream);
int dpgb_prod_virial_a_f64(double* virial, double* atom_virial,
                           const double* net_deriv, const double* env_deriv,
                           const double* rij, const int* nlist, int nloc,
                           int nall, int nnei, void* stream);
/* dpgb_prod_force_a_f64 without any device allocation.  No counterpart in
 * the reference.  For callers that cannot allocate device memory inside the
 * force call: an MD engine whose device memory belongs to its own pool
 * allocator, or an inner loop where cudaMalloc/cudaFree would synchronise
 * the whole device.  Same arguments and result as dpgb_prod_force_a_f64; the
 * scratch lives in one fixed 11 MiB device array of the library, so
 * nframes*nloc*nnei and nframes*nall must each be <= 262144 (larger sizes
 * return DPGB_EINVAL).  The first call on a device looks the array up
 * (cudaGetSymbolAddress) and should come before any stream capture; so
 * should the first call after the device's CUDA context changed (a reset
 * of the primary context, or a context of the caller's own), which looks
 * it up again.  All
 * calls share the array: calls that overlap on the GPU race, so serialise
 * them.  Synchronises the stream. */
int dpgb_prod_force_a_f64_noalloc(double* force, const double* net_deriv,
                                  const double* env_deriv, const int* nlist,
                                  int nloc, int nall, int nnei, int nframes,
                                  void* stream);

/* Second-order terms for force-loss training: replace
 * deepmd::prod_force_grad_a_gpu (source/lib/src/gpu/prod_force_grad.cu:
 * 10-57) and prod_virial_grad_a_gpu (prod_virial_grad.cu:14-52).
 *   grad [nf, nloc, 3] (force cotangent) / [9] (virial cotangent),
 *   grad_net [nf*nloc, 4*nnei]. */
int dpgb_prod_force_grad_a_f64(double* grad_net, const double* grad,
                               const double* env_deriv, const int* nlist,
                               int nloc, int nnei, int nframes, void* stream);
int dpgb_prod_virial_grad_a_f64(double* grad_net, const double* grad,
                                const double* env_deriv, const double* rij,
                                const int* nlist, int nloc, int nnei,
                                void* stream);

/* ------------------------------------------------------------------------
 * Plain tensor-core GEMM (no counterpart in the reference, whose kernels use
 * no tensor cores): D[M,N] (FP32, row-major) = A[M,K] . B[K,N] with A BF16
 * row-major and B given as Bt [N,K] BF16 row-major.  tcgen05.mma with TMEM
 * accumulators; N in 16..256 (multiple of 16), K a multiple of 16; device
 * pointers; synchronises the stream. */
int dpgb_tc_gemm_bf16(float* D, const void* A, const void* Bt, int M, int N,
                      int K, void* stream);

/* ------------------------------------------------------------------------
 * DeepPot: the whole se_e2_a energy / force / virial evaluation.
 * Mirrors the C API DP_NewDeepPot / DP_DeepPotCompute / DP_DeepPotComputeNList
 * (source/api_c/include/c_api.h:150,244-322) and the backend method
 * DeepPotBackend::computew (source/api_cc/include/DeepPot.h:14-200).
 *
 * The model is described by host pointers in the reference's own
 * parameterisation (descriptor mean/stddev [ntypes, nnei, 4]; per-net layer
 * matrices [num_in, num_out] row-major, biases, timesteps; fitting nets;
 * per-type energy bias) and copied to the device at creation. */
typedef struct dpgb_se_a_desc {
  int ntypes;
  int sel[DPGB_MAX_TYPES];
  double rcut, rcut_smth;
  int type_one_side;
  int n_emb;
  int emb_neuron[DPGB_MAX_LAYERS];
  int axis_neuron;
  int n_fit;
  int fit_neuron[DPGB_MAX_LAYERS];
  int dim_descrpt;
  const double* davg;
  const double* dstd;
  const double* emb_w[DPGB_MAX_TYPES * DPGB_MAX_TYPES][DPGB_MAX_LAYERS];
  const double* emb_b[DPGB_MAX_TYPES * DPGB_MAX_TYPES][DPGB_MAX_LAYERS];
  const double* emb_idt[DPGB_MAX_TYPES * DPGB_MAX_TYPES][DPGB_MAX_LAYERS];
  const double* fit_w[DPGB_MAX_TYPES][DPGB_MAX_LAYERS + 1];
  const double* fit_b[DPGB_MAX_TYPES][DPGB_MAX_LAYERS + 1];
  const double* fit_idt[DPGB_MAX_TYPES][DPGB_MAX_LAYERS + 1];
  const double* atom_ener_bias; /* [ntypes]: bias_atom_e + out_bias */
  const int* pair_mask;         /* [ntypes*ntypes] 1 keep, 0 excluded; or NULL */
  const double* table[DPGB_MAX_TYPES * DPGB_MAX_TYPES]; /* compressed nets */
  double table_info[DPGB_MAX_TYPES * DPGB_MAX_TYPES][6];
  int compressed;
} dpgb_se_a_desc;

/* Precision of a DeepPot evaluation. */
#define DPGB_PREC_FP64 0  /* plain FP64 throughout (the drop-in form) */
#define DPGB_PREC_MIXED 1 /* FP64 displacement, FP32 env matrix, tensor-core
                             embedding and fitting GEMMs in split BF16 (hi + lo
                             operands) with FP32 accumulation, FP64
                             energy/virial sums */

typedef struct dpgb_deeppot dpgb_deeppot;

/* Creates a model on the current CUDA device.  Returns NULL on failure
 * (message in dpgb_last_error()). */
dpgb_deeppot* dpgb_deeppot_new(const dpgb_se_a_desc* desc, int precision);

/* Frozen model files: the se_e2_a energy models that DeePMD-kit's PyTorch
 * backend freezes into a .pth TorchScript archive (`dp --pt freeze`, the
 * file DP_NewDeepPot(const char* model) takes: source/api_c/include/
 * c_api.h:150; DeepPotPT::init, source/api_cc/src/DeepPotPT.cc:73-152),
 * read on the host without libtorch: the configuration from the module's
 * model_def_script, the weights by their state-dict names, compressed
 * tables when the model was compressed.  content/size, when size > 0, is
 * the file's content (the reference's file_content argument) and path is
 * then not read.  Returns NULL on failure (dpgb_last_error()). */
typedef struct dpgb_model_file dpgb_model_file;
dpgb_model_file* dpgb_model_file_open(const char* path, const char* content,
                                      size_t size);
void dpgb_model_file_close(dpgb_model_file* m);
/* The model description (valid while m is open): pass to dpgb_deeppot_new. */
const dpgb_se_a_desc* dpgb_model_file_desc(const dpgb_model_file* m);
/* Space-separated element names of the types ("" when the model has none). */
const char* dpgb_model_file_type_map(const dpgb_model_file* m);
/* The model_def_script JSON text. */
const char* dpgb_model_file_config(const dpgb_model_file* m);
/* A weight by state-dict name: returns its element count (-1 if absent),
 * copies up to cap values (FP64) into out and, when ndim is set (in: the
 * capacity of shape, out: the rank), its shape into shape. */
long long dpgb_model_file_tensor(const dpgb_model_file* m, const char* name,
                                 double* out, long long cap, long long* shape,
                                 int* ndim);
void dpgb_deeppot_delete(dpgb_deeppot* dp);
/* Text of the last error stored on the handle, "" when the last call
 * succeeded (c_api.cc:2730 DP_DeepPotCheckOK). */
const char* dpgb_deeppot_check_ok(dpgb_deeppot* dp);

/* One or more frames of the same atom count with HOST buffers, as
 * DP_DeepPotCompute: coord [nframes, natom, 3], atype [natom] (shared by the
 * frames), box [nframes, 9] or NULL (open boundary).  Outputs (host, caller
 * allocated): energy [nframes], force [nframes, natom, 3], virial
 * [nframes, 9], atom_energy [nframes, natom] or NULL, atom_virial
 * [nframes, natom, 9] or NULL.  Copies in, evaluates, copies out and
 * synchronises its stream.  Page-locked (pinned) buffers are copied
 * directly, pageable ones through a pinned staging block.  Neighbour lists
 * are rebuilt every call (unless dpgb_deeppot_set_skin). */
int dpgb_deeppot_compute(dpgb_deeppot* dp, int nframes, int natom,
                         const double* coord, const int* atype,
                         const double* box, double* energy, double* force,
                         double* virial, double* atom_energy,
                         double* atom_virial);

/* The same with DEVICE coordinates and outputs on `stream`, without a final
 * synchronisation: the device-resident form used inside an MD loop.  The
 * atom types stay a HOST array (static metadata of the system; the type
 * grouping is cached across calls with identical types).  energy [nframes],
 * force [nframes, natom, 3], virial [nframes, 9], atom_energy, atom_virial
 * (optional) are FP64 device arrays. */
int dpgb_deeppot_compute_device(dpgb_deeppot* dp, int nframes, int natom,
                                const double* coord, const int* atype_host,
                                const double* box_host, double* energy,
                                double* force, double* virial,
                                double* atom_energy, double* atom_virial,
                                void* stream);

/* Neighbour-list reuse with a skin for periodic frames (both compute
 * forms above), the device-side counterpart of an MD code's Verlet list
 * (LAMMPS neigh_modify every/check yes) feeding DeepPot::compute's `ago`
 * (source/api_cc/src/DeepPotPT.cc:170-243; c_api.h:310-322).  skin > 0:
 * the candidates within rcut + skin are built on wrapped coordinates, and
 * rebuilt when `every` calls have passed since the last build or an atom
 * has moved more than skin / 2 since then (decided on the device; a new
 * box, atom count or type vector also rebuilds).  Between builds the
 * coordinates keep the build's wrap offsets and each call selects its list
 * at rcut from the candidates, in the order and with the truncation of a
 * fresh list.  skin = 0 (the default): a fresh list every call.  A
 * candidate row too narrow for the pairs within rcut + skin is an error of
 * that call (dpgb_deeppot_compute then widens the rows and repeats it
 * once; after dpgb_deeppot_compute_device, dpgb_deeppot_check_status
 * reports it and the next call widens and rebuilds). */
int dpgb_deeppot_set_skin(dpgb_deeppot* dp, double skin, int every);

/* CUDA-graph replay of the single-system evaluation (both compute forms,
 * periodic frames): with on = 1 the first call for a given shape, box and
 * set of buffers runs normally and captures the evaluation into a graph;
 * later calls with the same shape, box, buffers and handle state replay it
 * on the handle's stream (ordered after and before the caller's stream by
 * events) with no host-side work.  A change of any of them, or another
 * system computed on the handle, re-captures.  on = 0 (the default)
 * releases the graph. */
int dpgb_deeppot_set_graph(dpgb_deeppot* dp, int on);

/* Waits for `stream` (NULL: the stream of the last device-form evaluation,
 * else the handle's stream) and reports the
 * device-side errors of the last evaluation: neighbour overflow, skin
 * candidate truncation, a timed-out tensor-core wait.  The device form
 * (dpgb_deeppot_compute_device) does not synchronise, so its caller reads
 * these here. */
int dpgb_deeppot_check_status(dpgb_deeppot* dp, void* stream);

/* One frame with explicit ghost atoms and the caller's neighbour list, HOST
 * buffers: the DeepPot::compute(..., nghost, InputNlist, ago) path
 * (source/api_cc/src/DeepPotPT.cc:170-243) behind DP_DeepPotComputeNList
 * (source/api_c/include/c_api.h:310-322).  coord [nall, 3] and atype [nall]
 * with the nloc = nall - nghost local atoms first; the list is LAMMPS's
 * InputNlist: ilist [inum], numneigh [inum], firstneigh[inum][numneigh[ii]]
 * (indices in [0, nall), any order, may reach beyond rcut).  ago == 0 takes
 * the list afresh; ago > 0 reuses the stored list with the new coordinates.
 * Each call filters the list at rcut and orders it as forward_lower does
 * (by distance when a row is wider than sum(sel) or the model is
 * compressed, else the caller's order; then per type the first sel[t]).
 * Outputs: energy [1], virial [9], force [nall, 3] and atom_virial
 * [nall, 9] including the ghosts (the caller sums ghost entries back onto
 * their owners), atom_energy [nall] (0 on ghosts); box is not used. */
int dpgb_deeppot_compute_nlist(dpgb_deeppot* dp, int nall, int nghost,
                               const double* coord, const int* atype,
                               const double* box, int inum, const int* ilist,
                               const int* numneigh,
                               const int* const* firstneigh, int ago,
                               double* energy, double* force, double* virial,
                               double* atom_energy, double* atom_virial);

/* Batches of independent periodic frames of different sizes (no counterpart
 * in the reference, which evaluates frames one shape at a time,
 * deepmd/pt/infer/deep_eval.py): all frames go through one set of launches
 * — a cell list over the cells of every frame, the embedding over all
 * type-sorted atoms, the fitting per type over all frames — and the
 * evaluation can be captured in a CUDA graph and replayed.
 *   natoms [nframes], atype: the frames' types concatenated, box
 *   [nframes, 9] (every frame periodic; no face thinner than rcut / 2).
 * A batch borrows the handle's workspace: computing other systems with the
 * handle in between is allowed and makes the next batch call re-capture. */
typedef struct dpgb_batch dpgb_batch;
dpgb_batch* dpgb_batch_new(dpgb_deeppot* dp, int nframes, const int* natoms,
                           const int* atype, const double* box);
void dpgb_batch_delete(dpgb_batch* b);
int dpgb_batch_natoms(const dpgb_batch* b);
/* DEVICE buffers: coord [natoms, 3] (frames concatenated), energy
 * [nframes], force [natoms, 3], virial [nframes, 9].  use_graph: capture
 * the kernel sequence on the first call (after one plain evaluation) and
 * replay it while the buffer pointers, the stream and the handle's cached
 * state stay the same.  stream NULL = the handle's stream, synchronised. */
int dpgb_batch_compute_device(dpgb_batch* b, const double* coord,
                              double* energy, double* force, double* virial,
                              void* stream, int use_graph);
/* The same with HOST buffers (copies in and out, synchronises, reports
 * neighbour overflow). */
int dpgb_batch_compute(dpgb_batch* b, const double* coord, double* energy,
                       double* force, double* virial, int use_graph);

/* Size buckets of a batch and the work-item ("tile") size of each (no
 * counterpart in the reference; its launch-configuration tuner registry,
 * deepmd/kernels/autotune.py:1-87, is the precedent).  A frame of n atoms
 * is in bucket 0 (n <= 128), 1 (<= 512), 2 (<= 2048) or 3 (more).  The
 * persistent embedding / table kernels process the batch's rows in work
 * items of one centre type and one bucket; with tiles set, a bucket's rows
 * are cut into items of at most rows_per_item[k] rows (0: the default
 * split of about 3 x SMs items over all rows) and the CTAs draw the items,
 * largest first, from a device queue.  All zero (the default) = the
 * default split in a fixed stride.  Results do not depend on the tiles.
 * Setting different tiles makes the next evaluation re-cut the items and
 * re-capture its graph. */
#define DPGB_BATCH_BUCKETS 4
/* frames [4], atoms [4] (either may be NULL) */
int dpgb_batch_buckets(const dpgb_batch* b, int* frames, int* atoms);
/* rows_per_item [4], each 0 ... 2^20 */
int dpgb_batch_set_tiles(dpgb_batch* b, const int* rows_per_item);
int dpgb_batch_get_tiles(const dpgb_batch* b, int* rows_per_item);

/* The embedding stage of the mixed form on its own, behind the Python
 * DescrptSeA (deepmd/pt/model/descriptor/se_a.py:742-858; precision
 * "mixed"): the handle's tensor-core embedding — or, for a compressed
 * model, its fused FP32 table kernels — with the contraction to the
 * descriptor D = (G^T R~)^T (G^T R~)< / nnei^2, on per-frame extended atoms
 * and a formatted neighbour list, without the fitting.  DEVICE buffers on
 * `stream` (NULL: the legacy stream), no synchronisation:
 *   coord_ext [nf, nall, 3] FP64, atype_ext [nf, nall] (device), atype_loc
 *   [nloc] HOST (the local types, the same in every frame), nlist
 *   [nf, nloc, sum(sel)] (indices into the frame's extended atoms, type
 *   sections in the reference order, -1 padding)
 *   -> descrpt [nf, nloc, ng * axis] FP32, xyz [nf, nloc, 4, ng] FP32 (may
 *   be NULL; xyz[:, :, 1:4] is the reference's rot_mat transposed).
 * ticket (HOST, may be NULL) <- this forward's number.  The backward takes
 * dE/d descrpt [nf, nloc, ng * axis] FP32 to dE/d coord_ext [nf, nall, 3]
 * FP64 (every extended atom written) for the forward with that ticket, which
 * must be the handle's latest evaluation (else DPGB_EINVAL: its state is
 * gone).  FP64 handles return DPGB_EINVAL (their descriptor is the FP64
 * block). */
int dpgb_deeppot_descrpt_fwd(dpgb_deeppot* dp, int nf, int nloc, int nall,
                             const double* coord_ext, const int* atype_ext,
                             const int* atype_loc, const int* nlist,
                             float* descrpt, float* xyz,
                             unsigned long long* ticket, void* stream);
int dpgb_deeppot_descrpt_bwd(dpgb_deeppot* dp, unsigned long long ticket,
                             const float* g_descrpt, double* g_coord_ext,
                             void* stream);

/* Self-test of the bounded device-side waits (no counterpart in the
 * reference, which has no device-side waits of its own): one kernel waits
 * on an mbarrier that nothing completes, with a limit of limit_ms (0 < ...
 * <= 1000), gives up, records the timeout and ends.  Returns DPGB_ETIMEOUT
 * — the code a timed-out tensor-core wait gives every compute call — with
 * the CUDA context still usable; DPGB_OK would mean the wait did not run
 * out.  stream NULL = the legacy default stream; synchronises it. */
int dpgb_selftest_wait_timeout(double limit_ms, void* stream);

/* Number of kernel launches the last compute issued (for the benchmark). */
int dpgb_deeppot_last_launches(dpgb_deeppot* dp);

/* The neighbour list the last single-system evaluation built for itself,
 * for verification (no counterpart in the reference, where the list stays
 * inside DeepPot::compute: source/api_cc/src/DeepPotPT.cc:170-243).  HOST
 * buffers; waits for that evaluation to complete (on whichever stream it
 * ran):
 *   info [4]  <- nframes, natom, nnei (= sum(sel)), nshift (0 frames: the
 *                last evaluation had no list of its own — none yet, an
 *                external list or a batch; then the other pointers must be
 *                NULL);
 *   nlist [nframes * natom, nnei] <- extended indices e = s * natom + j
 *                (periodic image s of atom j; -1 padding), type sections of
 *                sel[t] in the reference order (deepmd/pt/utils/nlist.py);
 *   coord [nframes * natom, 3] <- the coordinates the list refers to
 *                (wrapped into the cell; with a skin, with the wrap offsets
 *                of the last candidate build);
 *   shift [nframes, nshift, 3] <- the Cartesian shift of each image s.
 * Any of nlist, coord, shift may be NULL. */
int dpgb_deeppot_last_nlist(dpgb_deeppot* dp, int* info, int* nlist,
                            double* coord, double* shift);

/* Stage timing with CUDA events on the compute stream (no counterpart in
 * the reference, whose DP_PROFILER hooks the libtorch profiler instead,
 * source/api_cc/src/DeepPotPT.cc:73-101).  set_profiling(1) creates the
 * events and clears the totals; after each compute, collect_stages()
 * waits for that call's events and adds its stage times; stage_times()
 * returns the totals in ms (DPGB_NUM_STAGES entries) and the number of
 * collected calls. */
#define DPGB_STAGE_NLIST 0     /* wrap + cell-list neighbour list */
#define DPGB_STAGE_TRANSPOSE 1 /* sorted transpose of the list */
#define DPGB_STAGE_DESC_FWD 2  /* env matrix + embedding + D */
#define DPGB_STAGE_FITTING 3   /* fitting forward + backward */
#define DPGB_STAGE_DESC_BWD 4  /* embedding recompute + backward + pair grads */
#define DPGB_STAGE_REDUCE 5    /* force gather, energy / virial sums */
#define DPGB_NUM_STAGES 6
int dpgb_deeppot_set_profiling(dpgb_deeppot* dp, int on);
int dpgb_deeppot_collect_stages(dpgb_deeppot* dp);
int dpgb_deeppot_stage_times(dpgb_deeppot* dp, double* ms, int* ncalls);

#ifdef __cplusplus
}
#endif
#endif
