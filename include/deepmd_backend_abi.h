/* The C++ interface a DeePMD-kit DeepPot backend plugin implements, declared
 * here so that the GB300 backend (deepmd-kit_gb300/plugin/deeppot_backend.cc)
 * builds without the reference's source tree.  A host built from the
 * reference (deepmd::DeepPot, DP_NewDeepPot) dlopens the plugin, calls the
 * factory symbols below and then the virtual methods through its own
 * declaration of these classes, so the virtual methods must sit in the same
 * order with the same parameter types as there:
 *   deepmd::DeepBaseModelBackend  source/api_cc/include/DeepBaseModel.h:13-84
 *   deepmd::DeepPotBackend        source/api_cc/include/DeepPot.h:14-375
 *   deepmd::InputNlist            source/lib/include/neighbor_list.h:20-57
 *   deepmd::deepmd_exception      source/lib/include/errors.h:11-16
 *   factory symbols and types     source/api_cc/include/BackendPlugin.h:19-72
 * (tests/test_plugin_abi.py compares the slot of every virtual method and
 * the field offsets of InputNlist with the reference's own headers). */
#pragma once

#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

namespace deepmd {

/* The error type hosts catch around backend calls. */
struct deepmd_exception : public std::runtime_error {
 public:
  deepmd_exception() : runtime_error("DeePMD-kit Error!") {}
  deepmd_exception(const std::string& msg) : runtime_error(std::string("DeePMD-kit Error: ") + msg) {}
};

/* A LAMMPS-style neighbour list as the host hands it over: ilist [inum],
 * numneigh [inum], firstneigh [inum][numneigh[ii]]; the communication fields
 * serve message-passing models only. */
struct InputNlist {
  int inum;
  int* ilist;
  int* numneigh;
  int** firstneigh;
  int nswap;
  int* sendnum;
  int* recvnum;
  int* firstrecv;
  int** sendlist;
  int* sendproc;
  int* recvproc;
  void* world;
  int mask = 0xFFFFFFFF;
  int* mapping = nullptr;
  int nprocs = 1;
  InputNlist()
      : inum(0), ilist(nullptr), numneigh(nullptr), firstneigh(nullptr), nswap(0), sendnum(nullptr),
        recvnum(nullptr), firstrecv(nullptr), sendlist(nullptr), sendproc(nullptr), recvproc(nullptr),
        world(nullptr) {}
  InputNlist(int inum_, int* ilist_, int* numneigh_, int** firstneigh_)
      : inum(inum_), ilist(ilist_), numneigh(numneigh_), firstneigh(firstneigh_), nswap(0), sendnum(nullptr),
        recvnum(nullptr), firstrecv(nullptr), sendlist(nullptr), sendproc(nullptr), recvproc(nullptr),
        world(nullptr) {}
};

class DeepBaseModelBackend {
 public:
  DeepBaseModelBackend() {}
  virtual ~DeepBaseModelBackend() {}
  virtual void init(const std::string& model, const int& gpu_rank = 0, const std::string& file_content = "") = 0;
  virtual double cutoff() const = 0;
  virtual int numb_types() const = 0;
  virtual int numb_types_spin() const = 0;
  virtual int dim_fparam() const = 0;
  virtual int dim_aparam() const = 0;
  virtual void get_type_map(std::string& type_map) = 0;
  virtual bool is_aparam_nall() const = 0;
  virtual bool has_default_fparam() const = 0;
};

class DeepPotBackend : public DeepBaseModelBackend {
 public:
  DeepPotBackend() {}
  virtual ~DeepPotBackend() {}
  virtual void init(const std::string& model, const int& gpu_rank = 0, const std::string& file_content = "") = 0;
  /* frames without a neighbour list: coord [nframes * natoms * 3], box
   * [nframes * 9] or empty (open boundary); outputs resized by the callee */
  virtual void computew(std::vector<double>& ener, std::vector<double>& force, std::vector<double>& virial,
                        std::vector<double>& atom_energy, std::vector<double>& atom_virial,
                        const std::vector<double>& coord, const std::vector<int>& atype,
                        const std::vector<double>& box, const std::vector<double>& fparam,
                        const std::vector<double>& aparam, const bool atomic) = 0;
  virtual void computew(std::vector<double>& ener, std::vector<float>& force, std::vector<float>& virial,
                        std::vector<float>& atom_energy, std::vector<float>& atom_virial,
                        const std::vector<float>& coord, const std::vector<int>& atype,
                        const std::vector<float>& box, const std::vector<float>& fparam,
                        const std::vector<float>& aparam, const bool atomic) = 0;
  /* one frame with nghost ghost atoms and the host's neighbour list; ago > 0
   * reuses the list of the last call with ago == 0 */
  virtual void computew(std::vector<double>& ener, std::vector<double>& force, std::vector<double>& virial,
                        std::vector<double>& atom_energy, std::vector<double>& atom_virial,
                        const std::vector<double>& coord, const std::vector<int>& atype,
                        const std::vector<double>& box, const int nghost, const InputNlist& inlist, const int& ago,
                        const std::vector<double>& fparam, const std::vector<double>& aparam,
                        const bool atomic) = 0;
  virtual void computew(std::vector<double>& ener, std::vector<float>& force, std::vector<float>& virial,
                        std::vector<float>& atom_energy, std::vector<float>& atom_virial,
                        const std::vector<float>& coord, const std::vector<int>& atype,
                        const std::vector<float>& box, const int nghost, const InputNlist& inlist, const int& ago,
                        const std::vector<float>& fparam, const std::vector<float>& aparam, const bool atomic) = 0;
  /* nframes frames, each with its own types: atype [nframes * natoms] */
  virtual void computew_mixed_type(std::vector<double>& ener, std::vector<double>& force,
                                   std::vector<double>& virial, std::vector<double>& atom_energy,
                                   std::vector<double>& atom_virial, const int& nframes,
                                   const std::vector<double>& coord, const std::vector<int>& atype,
                                   const std::vector<double>& box, const std::vector<double>& fparam,
                                   const std::vector<double>& aparam, const bool atomic) = 0;
  virtual void computew_mixed_type(std::vector<double>& ener, std::vector<float>& force,
                                   std::vector<float>& virial, std::vector<float>& atom_energy,
                                   std::vector<float>& atom_virial, const int& nframes,
                                   const std::vector<float>& coord, const std::vector<int>& atype,
                                   const std::vector<float>& box, const std::vector<float>& fparam,
                                   const std::vector<float>& aparam, const bool atomic) = 0;
  virtual int dim_chg_spin() const { return 0; }
  /* the same with a per-frame charge / spin vector, which models without
   * one ignore */
  virtual void computew(std::vector<double>& ener, std::vector<double>& force, std::vector<double>& virial,
                        std::vector<double>& atom_energy, std::vector<double>& atom_virial,
                        const std::vector<double>& coord, const std::vector<int>& atype,
                        const std::vector<double>& box, const std::vector<double>& fparam,
                        const std::vector<double>& aparam, const std::vector<double>& charge_spin,
                        const bool atomic) {
    computew(ener, force, virial, atom_energy, atom_virial, coord, atype, box, fparam, aparam, atomic);
  }
  virtual void computew(std::vector<double>& ener, std::vector<float>& force, std::vector<float>& virial,
                        std::vector<float>& atom_energy, std::vector<float>& atom_virial,
                        const std::vector<float>& coord, const std::vector<int>& atype,
                        const std::vector<float>& box, const std::vector<float>& fparam,
                        const std::vector<float>& aparam, const std::vector<double>& charge_spin,
                        const bool atomic) {
    computew(ener, force, virial, atom_energy, atom_virial, coord, atype, box, fparam, aparam, atomic);
  }
  virtual void computew(std::vector<double>& ener, std::vector<double>& force, std::vector<double>& virial,
                        std::vector<double>& atom_energy, std::vector<double>& atom_virial,
                        const std::vector<double>& coord, const std::vector<int>& atype,
                        const std::vector<double>& box, const int nghost, const InputNlist& inlist, const int& ago,
                        const std::vector<double>& fparam, const std::vector<double>& aparam,
                        const std::vector<double>& charge_spin, const bool atomic) {
    computew(ener, force, virial, atom_energy, atom_virial, coord, atype, box, nghost, inlist, ago, fparam, aparam,
             atomic);
  }
  virtual void computew(std::vector<double>& ener, std::vector<float>& force, std::vector<float>& virial,
                        std::vector<float>& atom_energy, std::vector<float>& atom_virial,
                        const std::vector<float>& coord, const std::vector<int>& atype,
                        const std::vector<float>& box, const int nghost, const InputNlist& inlist, const int& ago,
                        const std::vector<float>& fparam, const std::vector<float>& aparam,
                        const std::vector<double>& charge_spin, const bool atomic) {
    computew(ener, force, virial, atom_energy, atom_virial, coord, atype, box, nghost, inlist, ago, fparam, aparam,
             atomic);
  }
  virtual void computew_mixed_type(std::vector<double>& ener, std::vector<double>& force,
                                   std::vector<double>& virial, std::vector<double>& atom_energy,
                                   std::vector<double>& atom_virial, const int& nframes,
                                   const std::vector<double>& coord, const std::vector<int>& atype,
                                   const std::vector<double>& box, const std::vector<double>& fparam,
                                   const std::vector<double>& aparam, const std::vector<double>& charge_spin,
                                   const bool atomic) {
    computew_mixed_type(ener, force, virial, atom_energy, atom_virial, nframes, coord, atype, box, fparam, aparam,
                        atomic);
  }
  virtual void computew_mixed_type(std::vector<double>& ener, std::vector<float>& force,
                                   std::vector<float>& virial, std::vector<float>& atom_energy,
                                   std::vector<float>& atom_virial, const int& nframes,
                                   const std::vector<float>& coord, const std::vector<int>& atype,
                                   const std::vector<float>& box, const std::vector<float>& fparam,
                                   const std::vector<float>& aparam, const std::vector<double>& charge_spin,
                                   const bool atomic) {
    computew_mixed_type(ener, force, virial, atom_energy, atom_virial, nframes, coord, atype, box, fparam, aparam,
                        atomic);
  }
  /* graph-style device inputs of message-passing models; an se_e2_a backend
   * implements them by refusing */
  virtual void compute_edges_gpu(double* d_atom_energy, double* d_force, double* d_atom_virial,
                                 const double* d_coord, const int* d_atype, const int* d_edge_index,
                                 const double* d_edge_vec, const int nloc, const int nedge) = 0;
  virtual void compute_edges_gpu(double* d_atom_energy, double* d_force, double* d_atom_virial,
                                 const double* d_coord, const int* d_atype, const int* d_edge_index,
                                 const double* d_edge_vec, const int nloc, const int nedge,
                                 const std::vector<double>& fparam, const std::vector<double>& aparam,
                                 const int nall_nodes, const InputNlist* comm_nlist) = 0;
  virtual void compute_edges_gpu(double* d_atom_energy, double* d_force, double* d_atom_virial,
                                 const double* d_coord, const int* d_atype, const int* d_edge_index,
                                 const float* d_edge_vec, const int nloc, const int nedge,
                                 const std::vector<double>& fparam, const std::vector<double>& aparam,
                                 const int nall_nodes, const InputNlist* comm_nlist) = 0;
  virtual void compute_canonical_graph_gpu(double* d_atom_energy, double* d_force, double* d_atom_virial,
                                           const std::int64_t* d_atype, const std::int64_t* d_source,
                                           const float* d_edge_vec, const std::int64_t* d_destination_row_ptr,
                                           const std::int64_t* d_source_row_ptr,
                                           const std::int64_t* d_source_order, const int nloc,
                                           const int nall_nodes, const std::int64_t edge_storage) = 0;
  virtual bool supports_device_edge_inference() const = 0;
  virtual bool uses_fp32_edge_vectors() const = 0;
  virtual bool uses_canonical_graph_inference() const = 0;
};

}  // namespace deepmd

extern "C" {
/* Returns a deepmd::DeepPotBackend* as void* (NULL and a message in
 * *error_message, to be released by deepmd_free_backend_error_v1, on
 * failure); file_content / size, when size > 0, is the model file's content. */
void* deepmd_create_deeppot_backend_v1(const char* model, int gpu_rank, const char* file_content, std::size_t size,
                                       char** error_message);
void deepmd_delete_deeppot_backend_v1(void* backend);
void deepmd_free_backend_error_v1(char* error_message);
}
