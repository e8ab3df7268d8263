/* Test infrastructure only: the CPU oracle for the se_e2_a energy / force /
 * virial path.  A plain-C, FP64 restatement of the reference algorithm used
 * by tests/, __graft_entry__.smoke() and bench.py's CPU baseline leg as the
 * checker; the product never links it.  Each function names the reference
 * file:line it restates (paths relative to the deepmodeling/deepmd-kit tree).
 */
#ifndef DPGB_ORACLE_H
#define DPGB_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_MAX_TYPES 8
#define ORC_MAX_LAYERS 6

/* se_e2_a model in the reference's own parameterisation
 * (deepmd/pt/model/descriptor/se_a.py:477-576, task/ener.py, mlp.py:71-219).
 * Matrices are row-major [num_in, num_out] like MLPLayer.matrix.  Pointers of
 * absent parameters (idt without resnet_dt) are NULL. */
typedef struct orc_se_a_model {
  int ntypes;
  int sel[ORC_MAX_TYPES];
  double rcut, rcut_smth;
  int type_one_side;
  int n_emb;                          /* embedding layers */
  int emb_neuron[ORC_MAX_LAYERS];     /* widths, input width is 1 */
  int axis_neuron;
  int n_fit;                          /* hidden fitting layers */
  int fit_neuron[ORC_MAX_LAYERS];
  int dim_descrpt;                    /* emb_neuron[n_emb-1] * axis_neuron */
  const double* davg;                 /* [ntypes, nnei, 4] */
  const double* dstd;                 /* [ntypes, nnei, 4] */
  const double* emb_w[ORC_MAX_TYPES * ORC_MAX_TYPES][ORC_MAX_LAYERS];
  const double* emb_b[ORC_MAX_TYPES * ORC_MAX_TYPES][ORC_MAX_LAYERS];
  const double* emb_idt[ORC_MAX_TYPES * ORC_MAX_TYPES][ORC_MAX_LAYERS];
  const double* fit_w[ORC_MAX_TYPES][ORC_MAX_LAYERS + 1];
  const double* fit_b[ORC_MAX_TYPES][ORC_MAX_LAYERS + 1];
  const double* fit_idt[ORC_MAX_TYPES][ORC_MAX_LAYERS + 1];
  const double* atom_ener_bias;       /* [ntypes]: bias_atom_e + out_bias */
  const int* pair_mask;               /* [ntypes*ntypes] 1 keep / 0 exclude, or NULL */
  /* compressed embedding (tabulate_fusion_se_a), per net; NULL when plain */
  const double* table[ORC_MAX_TYPES * ORC_MAX_TYPES];
  double table_info[ORC_MAX_TYPES * ORC_MAX_TYPES][6];
  int compressed;
} orc_se_a_model;

/* ---- tabulate_fusion_se_a (source/lib/src/tabulate.cc:162-449) ---- */
void orc_tabulate_fusion_se_a_f64(double* out, const double* table,
                                  const double* info, const double* em_x,
                                  const double* em, int nloc, int nnei,
                                  int last_layer_size, int is_sorted);
void orc_tabulate_fusion_se_a_f32(float* out, const float* table,
                                  const float* info, const float* em_x,
                                  const float* em, int nloc, int nnei,
                                  int last_layer_size, int is_sorted);
void orc_tabulate_fusion_se_a_grad_f64(double* dy_dem_x, double* dy_dem,
                                       const double* table, const double* info,
                                       const double* em_x, const double* em,
                                       const double* dy, int nloc, int nnei,
                                       int last_layer_size, int is_sorted);
void orc_tabulate_fusion_se_a_grad_f32(float* dy_dem_x, float* dy_dem,
                                       const float* table, const float* info,
                                       const float* em_x, const float* em,
                                       const float* dy, int nloc, int nnei,
                                       int last_layer_size, int is_sorted);
void orc_tabulate_fusion_se_a_grad_grad_f64(
    double* dz_dy, const double* table, const double* info, const double* em_x,
    const double* em, const double* dz_dy_dem_x, const double* dz_dy_dem,
    int nloc, int nnei, int last_layer_size, int is_sorted);
void orc_tabulate_fusion_se_a_grad_grad_f32(
    float* dz_dy, const float* table, const float* info, const float* em_x,
    const float* em, const float* dz_dy_dem_x, const float* dz_dy_dem,
    int nloc, int nnei, int last_layer_size, int is_sorted);

/* ---- neighbour lists ---- */
/* C++ order: (type, fp32 r^2, index), truncated per type to sel
 * (source/lib/src/fmt_nlist.cc:98-150).  in_rows: dense [nloc, max_nbor]
 * candidate rows with counts.  Returns the number of rows that overflowed. */
int orc_format_nlist_cpp(int* nlist, const double* coord, const int* atype,
                         const int* in_rows, const int* in_counts, int max_nbor,
                         int nloc, int nall, double rcut, const int* sel,
                         int ntypes);
/* PyTorch order (deepmd/pt/utils/nlist.py:49-199,304-337): all extended
 * atoms within rcut ordered by (fp64 distance, extended index), the nearest
 * sum(sel) kept, then split per type keeping the first sel[t].  A binned
 * search over the extended atoms.  Returns 0. */
int orc_build_nlist_pt(int* nlist, const double* coord_ext, const int* atype_ext,
                       int nloc, int nall, double rcut, const int* sel,
                       int ntypes);

/* ---- env matrix (source/lib/src/env_mat.cc:123-223 + prod_env_mat.cc:14-132)
 * em [nloc, nnei, 4] normalised, em_deriv [nloc, nnei, 4, 3] (derivative with
 * respect to the centre atom, divided by std), rij [nloc, nnei, 3].  As in the
 * reference, the switching radii are used as floats. */
void orc_env_mat_a(double* em, double* em_deriv, double* rij,
                   const double* coord_ext, const int* atype_ext,
                   const int* nlist, const double* davg, const double* dstd,
                   int nloc, int nnei, double rcut, double rcut_smth);

/* ---- force / virial (source/lib/src/prod_force.cc:23-87,
 * prod_virial.cc:22-69, prod_force_grad.cc, prod_virial_grad.cc) ---- */
void orc_prod_force_a(double* force, const double* net_deriv,
                      const double* env_deriv, const int* nlist, int nloc,
                      int nall, int nnei);
void orc_prod_virial_a(double* virial, double* atom_virial,
                       const double* net_deriv, const double* env_deriv,
                       const double* rij, const int* nlist, int nloc, int nall,
                       int nnei);
void orc_prod_force_grad_a(double* grad_net, const double* grad,
                           const double* env_deriv, const int* nlist, int nloc,
                           int nnei);
void orc_prod_virial_grad_a(double* grad_net, const double* grad,
                            const double* env_deriv, const double* rij,
                            const int* nlist, int nloc, int nnei);

/* ---- the full se_e2_a energy / force / virial of one frame (plain FP64, or
 * the FP64 table form when model->compressed).  Restates
 * DescrptBlockSeA.forward (se_a.py:742-858), the energy fitting
 * (task/fitting.py:734-899) and the autograd force/virial
 * (model/transform_output.py:68-99,155-209).  Outputs on extended atoms:
 * force_ext [nall,3], atom_virial_ext [nall,9]; atom_energy [nloc];
 * virial [9]; descriptor [nloc, dim_descrpt] and rot_mat [nloc, ng, 3] when
 * non-NULL.  Returns 0. */
int orc_se_a_energy_force(const orc_se_a_model* model, const double* coord_ext,
                          const int* atype_ext, const int* nlist, int nloc,
                          int nall, double* atom_energy, double* force_ext,
                          double* virial, double* atom_virial_ext,
                          double* descriptor, double* rot_mat);

int orc_num_threads(void);

#ifdef __cplusplus
}
#endif
#endif
