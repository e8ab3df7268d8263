// Test infrastructure only: a C-ABI shim around the reference's own CPU
// library (source/lib/src/*.cc of deepmodeling/deepmd-kit), compiled from the
// reference sources where they lie by oracle/build_ref.sh into oracle/_ref/.
// It is the checker for the restated oracle (oracle/dpgb_oracle.c) and for the
// CUDA library; nothing in the product links or loads it.
//
// Every entry point forwards plain pointers to the reference function named in
// its comment (file:line of the reference header/source).
#include <cstring>
#include <vector>

#include "coord.h"
#include "env_mat.h"
#include "fmt_nlist.h"
#include "neighbor_list.h"
#include "prod_env_mat.h"
#include "prod_force.h"
#include "prod_force_grad.h"
#include "prod_virial.h"
#include "prod_virial_grad.h"
#include "region.h"
#include "tabulate.h"
#include "SimulationRegion.h"

namespace {

// Dense [nrow, max_nbor] neighbour rows (+counts) -> the reference's
// LAMMPS-style InputNlist (source/lib/include/neighbor_list.h:15-119).
struct DenseNlist {
  std::vector<int> ilist, numneigh;
  std::vector<int*> firstneigh;
  std::vector<int> storage;
  deepmd::InputNlist in;
  DenseNlist(const int* rows, const int* counts, int nrow, int max_nbor)
      : ilist(nrow), numneigh(nrow), firstneigh(nrow),
        storage(rows, rows + (size_t)nrow * max_nbor) {
    for (int ii = 0; ii < nrow; ++ii) {
      ilist[ii] = ii;
      numneigh[ii] = counts[ii];
      firstneigh[ii] = storage.data() + (size_t)ii * max_nbor;
    }
    in = deepmd::InputNlist(nrow, ilist.data(), numneigh.data(),
                            firstneigh.data());
  }
};

std::vector<int> make_sec(const int* sel, int ntypes) {
  std::vector<int> sec(ntypes + 1, 0);
  for (int ii = 0; ii < ntypes; ++ii) sec[ii + 1] = sec[ii] + sel[ii];
  return sec;
}

}  // namespace

extern "C" {

// source/lib/include/tabulate.h:29 tabulate_fusion_se_a_cpu
int ref_tabulate_fusion_se_a_f64(double* out, const double* table,
                                 const double* info, const double* em_x,
                                 const double* em, int nloc, int nnei,
                                 int last_layer_size, int is_sorted) {
  deepmd::tabulate_fusion_se_a_cpu<double>(out, table, info, em_x, em, nullptr,
                                           nloc, nnei, last_layer_size,
                                           is_sorted != 0, 4);
  return 0;
}
int ref_tabulate_fusion_se_a_f32(float* out, const float* table,
                                 const float* info, const float* em_x,
                                 const float* em, int nloc, int nnei,
                                 int last_layer_size, int is_sorted) {
  deepmd::tabulate_fusion_se_a_cpu<float>(out, table, info, em_x, em, nullptr,
                                          nloc, nnei, last_layer_size,
                                          is_sorted != 0, 4);
  return 0;
}
// source/lib/include/tabulate.h:43 tabulate_fusion_se_a_grad_cpu
int ref_tabulate_fusion_se_a_grad_f64(double* dy_dem_x, double* dy_dem,
                                      const double* table, const double* info,
                                      const double* em_x, const double* em,
                                      const double* dy, int nloc, int nnei,
                                      int last_layer_size, int is_sorted) {
  deepmd::tabulate_fusion_se_a_grad_cpu<double>(
      dy_dem_x, dy_dem, nullptr, table, info, em_x, em, nullptr, dy, nloc,
      nnei, last_layer_size, is_sorted != 0, 4);
  return 0;
}
int ref_tabulate_fusion_se_a_grad_f32(float* dy_dem_x, float* dy_dem,
                                      const float* table, const float* info,
                                      const float* em_x, const float* em,
                                      const float* dy, int nloc, int nnei,
                                      int last_layer_size, int is_sorted) {
  deepmd::tabulate_fusion_se_a_grad_cpu<float>(
      dy_dem_x, dy_dem, nullptr, table, info, em_x, em, nullptr, dy, nloc,
      nnei, last_layer_size, is_sorted != 0, 4);
  return 0;
}
// source/lib/include/tabulate.h:59 tabulate_fusion_se_a_grad_grad_cpu
int ref_tabulate_fusion_se_a_grad_grad_f64(
    double* dz_dy, const double* table, const double* info, const double* em_x,
    const double* em, const double* dz_dy_dem_x, const double* dz_dy_dem,
    int nloc, int nnei, int last_layer_size, int is_sorted) {
  deepmd::tabulate_fusion_se_a_grad_grad_cpu<double>(
      dz_dy, table, info, em_x, em, nullptr, dz_dy_dem_x, dz_dy_dem, nullptr,
      nloc, nnei, last_layer_size, is_sorted != 0, 4);
  return 0;
}
int ref_tabulate_fusion_se_a_grad_grad_f32(
    float* dz_dy, const float* table, const float* info, const float* em_x,
    const float* em, const float* dz_dy_dem_x, const float* dz_dy_dem,
    int nloc, int nnei, int last_layer_size, int is_sorted) {
  deepmd::tabulate_fusion_se_a_grad_grad_cpu<float>(
      dz_dy, table, info, em_x, em, nullptr, dz_dy_dem_x, dz_dy_dem, nullptr,
      nloc, nnei, last_layer_size, is_sorted != 0, 4);
  return 0;
}

// source/lib/include/prod_env_mat.h:11 prod_env_mat_a_cpu (one frame)
int ref_prod_env_mat_a_f64(double* em, double* em_deriv, double* rij,
                           int* nlist, const double* coord, const int* type,
                           const int* in_rows, const int* in_counts,
                           int max_nbor, const double* avg, const double* std,
                           int nloc, int nall, double rcut, double rcut_smth,
                           const int* sel, int ntypes) {
  DenseNlist dn(in_rows, in_counts, nloc, max_nbor);
  std::vector<int> sec = make_sec(sel, ntypes);
  deepmd::prod_env_mat_a_cpu<double>(em, em_deriv, rij, nlist, coord, type,
                                     dn.in, max_nbor, avg, std, nloc, nall,
                                     (float)rcut, (float)rcut_smth, sec);
  return 0;
}
int ref_prod_env_mat_a_f32(float* em, float* em_deriv, float* rij, int* nlist,
                           const float* coord, const int* type,
                           const int* in_rows, const int* in_counts,
                           int max_nbor, const float* avg, const float* std,
                           int nloc, int nall, double rcut, double rcut_smth,
                           const int* sel, int ntypes) {
  DenseNlist dn(in_rows, in_counts, nloc, max_nbor);
  std::vector<int> sec = make_sec(sel, ntypes);
  deepmd::prod_env_mat_a_cpu<float>(em, em_deriv, rij, nlist, coord, type,
                                    dn.in, max_nbor, avg, std, nloc, nall,
                                    (float)rcut, (float)rcut_smth, sec);
  return 0;
}

// source/lib/include/fmt_nlist.h:12 format_nlist_cpu
int ref_format_nlist_f64(int* nlist, const double* coord, const int* type,
                         const int* in_rows, const int* in_counts,
                         int max_nbor, int nloc, int nall, double rcut,
                         const int* sel, int ntypes) {
  DenseNlist dn(in_rows, in_counts, nloc, max_nbor);
  std::vector<int> sec = make_sec(sel, ntypes);
  deepmd::format_nlist_cpu<double>(nlist, dn.in, coord, type, nloc, nall,
                                   (float)rcut, sec);
  return 0;
}

// source/lib/include/prod_force.h:19 prod_force_a_cpu
int ref_prod_force_a_f64(double* force, const double* net_deriv,
                         const double* env_deriv, const int* nlist, int nloc,
                         int nall, int nnei, int nframes) {
  deepmd::prod_force_a_cpu<double>(force, net_deriv, env_deriv, nlist, nloc,
                                   nall, nnei, nframes);
  return 0;
}
// source/lib/include/prod_virial.h:6 prod_virial_a_cpu
int ref_prod_virial_a_f64(double* virial, double* atom_virial,
                          const double* net_deriv, const double* env_deriv,
                          const double* rij, const int* nlist, int nloc,
                          int nall, int nnei) {
  deepmd::prod_virial_a_cpu<double>(virial, atom_virial, net_deriv, env_deriv,
                                    rij, nlist, nloc, nall, nnei);
  return 0;
}
// source/lib/include/prod_force_grad.h:7 prod_force_grad_a_cpu
int ref_prod_force_grad_a_f64(double* grad_net, const double* grad,
                              const double* env_deriv, const int* nlist,
                              int nloc, int nnei, int nframes) {
  deepmd::prod_force_grad_a_cpu<double>(grad_net, grad, env_deriv, nlist, nloc,
                                        nnei, nframes);
  return 0;
}
// source/lib/include/prod_virial_grad.h:7 prod_virial_grad_a_cpu
int ref_prod_virial_grad_a_f64(double* grad_net, const double* grad,
                               const double* env_deriv, const double* rij,
                               const int* nlist, int nloc, int nnei) {
  deepmd::prod_virial_grad_a_cpu<double>(grad_net, grad, env_deriv, rij, nlist,
                                         nloc, nnei);
  return 0;
}

// Legacy periodic copy + grid neighbour list used by the reference's own unit
// tests (source/lib/include/neighbor_list.h:300-352).  Writes the extended
// coordinates/types/mapping and the dense neighbour rows of the first nloc
// atoms into caller buffers of capacity mem_nall / mem_nbor.  Returns nall, or
// -1 when a buffer is too small.
int ref_copy_coord_build_nlist(double* out_c, int* out_t, int* mapping,
                               int* rows, int* counts, int mem_nall,
                               int mem_nbor, const double* in_c,
                               const int* in_t, int nloc, const double* box,
                               double rc) {
  SimulationRegion<double> region;
  double boxv[9];
  std::memcpy(boxv, box, sizeof(boxv));
  region.reinitBox(boxv);
  std::vector<double> posi(in_c, in_c + 3 * nloc), posi_cpy;
  std::vector<int> atype(in_t, in_t + nloc), atype_cpy, map, ncell, ngcell;
  copy_coord(posi_cpy, atype_cpy, map, ncell, ngcell, posi, atype, rc, region);
  const int nall = (int)posi_cpy.size() / 3;
  if (nall > mem_nall) return -1;
  std::vector<int> nat_stt(3, 0), ext_stt(3), ext_end(3);
  for (int dd = 0; dd < 3; ++dd) {
    ext_stt[dd] = -ngcell[dd];
    ext_end[dd] = ncell[dd] + ngcell[dd];
  }
  std::vector<std::vector<int> > nlist_a, nlist_r;
  build_nlist(nlist_a, nlist_r, posi_cpy, nloc, rc, rc, nat_stt, ncell,
              ext_stt, ext_end, region, ncell);
  std::memcpy(out_c, posi_cpy.data(), sizeof(double) * 3 * nall);
  std::memcpy(out_t, atype_cpy.data(), sizeof(int) * nall);
  std::memcpy(mapping, map.data(), sizeof(int) * nall);
  for (int ii = 0; ii < nloc; ++ii) {
    const int nn = (int)nlist_a[ii].size();
    if (nn > mem_nbor) return -1;
    counts[ii] = nn;
    for (int jj = 0; jj < mem_nbor; ++jj)
      rows[(size_t)ii * mem_nbor + jj] = jj < nn ? nlist_a[ii][jj] : -1;
  }
  return nall;
}

// source/lib/include/coord.h:25 copy_coord_cpu + neighbor_list.h:167
// build_nlist_cpu: the reference's cell-map ghost copy and its O(N^2) list.
int ref_copy_coord_cpu_build_nlist_cpu(double* out_c, int* out_t, int* mapping,
                                       int* rows, int* counts, int mem_nall,
                                       int mem_nbor, const double* in_c,
                                       const int* in_t, int nloc,
                                       const double* box, double rc) {
  double boxt[9], rec[9];
  std::memcpy(boxt, box, sizeof(boxt));
  deepmd::Region<double> region(boxt, rec);
  deepmd::init_region_cpu(region, boxt);
  int nall = 0;
  int ret = deepmd::copy_coord_cpu<double>(out_c, out_t, mapping, &nall, in_c,
                                           in_t, nloc, mem_nall, (float)rc,
                                           region);
  if (ret != 0) return -1;
  std::vector<int> ilist(nloc), numneigh(nloc);
  std::vector<int*> firstneigh(nloc);
  for (int ii = 0; ii < nloc; ++ii)
    firstneigh[ii] = rows + (size_t)ii * mem_nbor;
  deepmd::InputNlist in(nloc, ilist.data(), numneigh.data(), firstneigh.data());
  int max_list = 0;
  ret = deepmd::build_nlist_cpu<double>(in, &max_list, out_c, nloc, nall,
                                        mem_nbor, (float)rc, 1, out_t);
  if (ret != 0) return -1;
  for (int ii = 0; ii < nloc; ++ii) {
    counts[ii] = numneigh[ii];
    for (int jj = numneigh[ii]; jj < mem_nbor; ++jj)
      rows[(size_t)ii * mem_nbor + jj] = -1;
  }
  return nall;
}

}  // extern "C"
