// Test probe (not shipped): prints the vtable slot of every virtual method of
// deepmd::DeepPotBackend and the field offsets of deepmd::InputNlist, as the
// header given at compile time declares them.  Built twice by
// tests/test_plugin_abi.py -- once against the reference's own headers, once
// against include/deepmd_backend_abi.h -- and the two outputs must agree.
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#ifdef PROBE_REFERENCE
#include "DeepPot.h"
#else
#include "deepmd_backend_abi.h"
#endif

using deepmd::DeepPotBackend;
using deepmd::InputNlist;
using VD = std::vector<double>;
using VF = std::vector<float>;
using VI = std::vector<int>;

// Itanium C++ ABI: a pointer to a virtual member function holds 1 + the
// byte offset of its vtable slot
template <typename T>
long slot(T pmf) {
  struct {
    std::uintptr_t ptr, adj;
  } r;
  static_assert(sizeof(pmf) == sizeof(r), "unexpected member pointer size");
  std::memcpy(&r, &pmf, sizeof(r));
  return (r.ptr & 1) ? (long)((r.ptr - 1) / sizeof(void*)) : -1;
}


int main() {
  std::printf("%-40s %ld\n", "init", slot(&DeepPotBackend::init));
  std::printf("%-40s %ld\n", "cutoff", slot(&DeepPotBackend::cutoff));
  std::printf("%-40s %ld\n", "numb_types", slot(&DeepPotBackend::numb_types));
  std::printf("%-40s %ld\n", "numb_types_spin", slot(&DeepPotBackend::numb_types_spin));
  std::printf("%-40s %ld\n", "dim_fparam", slot(&DeepPotBackend::dim_fparam));
  std::printf("%-40s %ld\n", "dim_aparam", slot(&DeepPotBackend::dim_aparam));
  std::printf("%-40s %ld\n", "get_type_map", slot(&DeepPotBackend::get_type_map));
  std::printf("%-40s %ld\n", "is_aparam_nall", slot(&DeepPotBackend::is_aparam_nall));
  std::printf("%-40s %ld\n", "has_default_fparam", slot(&DeepPotBackend::has_default_fparam));
  using C1 = void (DeepPotBackend::*)(VD&, VD&, VD&, VD&, VD&, const VD&, const VI&, const VD&, const VD&, const VD&,
                                      const bool);
  using C2 = void (DeepPotBackend::*)(VD&, VF&, VF&, VF&, VF&, const VF&, const VI&, const VF&, const VF&, const VF&,
                                      const bool);
  using C3 = void (DeepPotBackend::*)(VD&, VD&, VD&, VD&, VD&, const VD&, const VI&, const VD&, const int,
                                      const InputNlist&, const int&, const VD&, const VD&, const bool);
  using C4 = void (DeepPotBackend::*)(VD&, VF&, VF&, VF&, VF&, const VF&, const VI&, const VF&, const int,
                                      const InputNlist&, const int&, const VF&, const VF&, const bool);
  using M1 = void (DeepPotBackend::*)(VD&, VD&, VD&, VD&, VD&, const int&, const VD&, const VI&, const VD&, const VD&,
                                      const VD&, const bool);
  using M2 = void (DeepPotBackend::*)(VD&, VF&, VF&, VF&, VF&, const int&, const VF&, const VI&, const VF&, const VF&,
                                      const VF&, const bool);
  using Q1 = void (DeepPotBackend::*)(VD&, VD&, VD&, VD&, VD&, const VD&, const VI&, const VD&, const VD&, const VD&,
                                      const VD&, const bool);
  using Q2 = void (DeepPotBackend::*)(VD&, VF&, VF&, VF&, VF&, const VF&, const VI&, const VF&, const VF&, const VF&,
                                      const VD&, const bool);
  using Q3 = void (DeepPotBackend::*)(VD&, VD&, VD&, VD&, VD&, const VD&, const VI&, const VD&, const int,
                                      const InputNlist&, const int&, const VD&, const VD&, const VD&, const bool);
  using Q4 = void (DeepPotBackend::*)(VD&, VF&, VF&, VF&, VF&, const VF&, const VI&, const VF&, const int,
                                      const InputNlist&, const int&, const VF&, const VF&, const VD&, const bool);
  using N1 = void (DeepPotBackend::*)(VD&, VD&, VD&, VD&, VD&, const int&, const VD&, const VI&, const VD&, const VD&,
                                      const VD&, const VD&, const bool);
  using N2 = void (DeepPotBackend::*)(VD&, VF&, VF&, VF&, VF&, const int&, const VF&, const VI&, const VF&, const VF&,
                                      const VF&, const VD&, const bool);
  using E1 = void (DeepPotBackend::*)(double*, double*, double*, const double*, const int*, const int*, const double*,
                                      const int, const int);
  using E2 = void (DeepPotBackend::*)(double*, double*, double*, const double*, const int*, const int*, const double*,
                                      const int, const int, const VD&, const VD&, const int, const InputNlist*);
  using E3 = void (DeepPotBackend::*)(double*, double*, double*, const double*, const int*, const int*, const float*,
                                      const int, const int, const VD&, const VD&, const int, const InputNlist*);
  std::printf("%-40s %ld\n", "computew double", slot(static_cast<C1>(&DeepPotBackend::computew)));
  std::printf("%-40s %ld\n", "computew float", slot(static_cast<C2>(&DeepPotBackend::computew)));
  std::printf("%-40s %ld\n", "computew nlist double", slot(static_cast<C3>(&DeepPotBackend::computew)));
  std::printf("%-40s %ld\n", "computew nlist float", slot(static_cast<C4>(&DeepPotBackend::computew)));
  std::printf("%-40s %ld\n", "computew_mixed_type double", slot(static_cast<M1>(&DeepPotBackend::computew_mixed_type)));
  std::printf("%-40s %ld\n", "computew_mixed_type float", slot(static_cast<M2>(&DeepPotBackend::computew_mixed_type)));
  std::printf("%-40s %ld\n", "dim_chg_spin", slot(&DeepPotBackend::dim_chg_spin));
  std::printf("%-40s %ld\n", "computew chg_spin double", slot(static_cast<Q1>(&DeepPotBackend::computew)));
  std::printf("%-40s %ld\n", "computew chg_spin float", slot(static_cast<Q2>(&DeepPotBackend::computew)));
  std::printf("%-40s %ld\n", "computew nlist chg_spin double", slot(static_cast<Q3>(&DeepPotBackend::computew)));
  std::printf("%-40s %ld\n", "computew nlist chg_spin float", slot(static_cast<Q4>(&DeepPotBackend::computew)));
  std::printf("%-40s %ld\n", "mixed_type chg_spin double", slot(static_cast<N1>(&DeepPotBackend::computew_mixed_type)));
  std::printf("%-40s %ld\n", "mixed_type chg_spin float", slot(static_cast<N2>(&DeepPotBackend::computew_mixed_type)));
  std::printf("%-40s %ld\n", "compute_edges_gpu 1", slot(static_cast<E1>(&DeepPotBackend::compute_edges_gpu)));
  std::printf("%-40s %ld\n", "compute_edges_gpu 2", slot(static_cast<E2>(&DeepPotBackend::compute_edges_gpu)));
  std::printf("%-40s %ld\n", "compute_edges_gpu 3", slot(static_cast<E3>(&DeepPotBackend::compute_edges_gpu)));
  std::printf("%-40s %ld\n", "compute_canonical_graph_gpu", slot(&DeepPotBackend::compute_canonical_graph_gpu));
  std::printf("%-40s %ld\n", "supports_device_edge_inference", slot(&DeepPotBackend::supports_device_edge_inference));
  std::printf("%-40s %ld\n", "uses_fp32_edge_vectors", slot(&DeepPotBackend::uses_fp32_edge_vectors));
  std::printf("%-40s %ld\n", "uses_canonical_graph_inference", slot(&DeepPotBackend::uses_canonical_graph_inference));
  std::printf("%-40s %zu\n", "InputNlist size", sizeof(InputNlist));
  std::printf("%-40s %zu %zu %zu %zu\n", "InputNlist inum ilist numneigh firstneigh", offsetof(InputNlist, inum),
              offsetof(InputNlist, ilist), offsetof(InputNlist, numneigh), offsetof(InputNlist, firstneigh));
  std::printf("%-40s %zu %zu %zu\n", "InputNlist mask mapping nprocs", offsetof(InputNlist, mask),
              offsetof(InputNlist, mapping), offsetof(InputNlist, nprocs));
  return 0;
}
