// DeePMD-kit DeepPot backend plugin on the GB300 kernels of libdpgb.
//
// A host built from the reference (deepmd::DeepPot::init, source/api_cc/src/
// DeepPot.cc:26-42; the C API DP_NewDeepPot, source/api_c/include/c_api.h:150)
// picks a backend by the model file's suffix and dlopens its plugin
// library (source/api_cc/src/BackendPlugin.cc: lib<name>.so from
// DP_BACKEND_PLUGIN_PATH or next to libdeepmd_cc; the PyTorch backend's name
// for .pth files is deepmd_backend_pt).  This library exports the plugin's
// three C symbols and implements deepmd::DeepPotBackend for se_e2_a energy
// models: the frozen .pth is read by dpgb_model_file_open (no libtorch),
// the evaluation runs in dpgb_deeppot_compute / dpgb_deeppot_compute_nlist.
//
// Semantics follow the reference PyTorch backend (DeepPotPT::compute,
// source/api_cc/src/DeepPotPT.cc:155-378): outputs are resized by the
// backend; without a list coord is [nframes * natoms * 3] with box
// [nframes * 9] or empty (open boundary); with a list the force and atomic
// virial cover all nall atoms (the host folds ghosts back).  Frame and
// atomic parameters are refused (se_e2_a energy models have none).
// Environment: DP_GB300_PRECISION=mixed selects the mixed-precision form
// (default: the FP64 form).  The device is gpu_rank modulo the GPU count.
#include <cuda_runtime.h>

#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "deepmd_backend_abi.h"
#include "dpgb.h"

namespace {

[[noreturn]] void raise(const std::string& what) { throw deepmd::deepmd_exception(what); }

void check(int rc, dpgb_deeppot* dp = nullptr) {
  if (rc == DPGB_OK) return;
  std::string msg = dp ? dpgb_deeppot_check_ok(dp) : "";
  if (msg.empty()) msg = dpgb_last_error();
  raise("GB300 backend: " + msg);
}

template <typename V>
std::vector<double> to_double(const std::vector<V>& v) {
  return std::vector<double>(v.begin(), v.end());
}
template <typename V>
void from_double(std::vector<V>& out, const std::vector<double>& v) {
  out.assign(v.begin(), v.end());
}

class DeepPotGB300 final : public deepmd::DeepPotBackend {
 public:
  ~DeepPotGB300() override {
    if (dp_) {
      cudaSetDevice(device_);
      dpgb_deeppot_delete(dp_);
    }
  }

  void init(const std::string& model, const int& gpu_rank, const std::string& file_content) override {
    int ngpu = 0;
    if (cudaGetDeviceCount(&ngpu) != cudaSuccess || ngpu <= 0) raise("GB300 backend: no CUDA device");
    device_ = (gpu_rank < 0 ? 0 : gpu_rank) % ngpu;
    if (cudaSetDevice(device_) != cudaSuccess) raise("GB300 backend: cannot select the CUDA device");
    dpgb_model_file* mf = dpgb_model_file_open(model.c_str(), file_content.data(), file_content.size());
    if (!mf) raise(std::string("GB300 backend: ") + dpgb_last_error());
    const dpgb_se_a_desc* d = dpgb_model_file_desc(mf);
    rcut_ = d->rcut;
    ntypes_ = d->ntypes;
    type_map_ = dpgb_model_file_type_map(mf);
    const char* prec = std::getenv("DP_GB300_PRECISION");
    const int precision = prec && std::strcmp(prec, "mixed") == 0 ? DPGB_PREC_MIXED : DPGB_PREC_FP64;
    dp_ = dpgb_deeppot_new(d, precision);
    dpgb_model_file_close(mf);
    if (!dp_) raise(std::string("GB300 backend: ") + dpgb_last_error());
  }

  double cutoff() const override { return rcut_; }
  int numb_types() const override { return ntypes_; }
  int numb_types_spin() const override { return 0; }
  int dim_fparam() const override { return 0; }
  int dim_aparam() const override { return 0; }
  void get_type_map(std::string& type_map) override { type_map = type_map_; }
  bool is_aparam_nall() const override { return false; }
  bool has_default_fparam() const override { return false; }

  // ---- frames without a neighbour list
  void computew(std::vector<double>& ener, std::vector<double>& force, std::vector<double>& virial,
                std::vector<double>& atom_energy, std::vector<double>& atom_virial, const std::vector<double>& coord,
                const std::vector<int>& atype, const std::vector<double>& box, const std::vector<double>& fparam,
                const std::vector<double>& aparam, const bool atomic) override {
    frames(ener, force, virial, atom_energy, atom_virial, coord, atype, box, fparam.size() + aparam.size(), atomic);
  }
  void computew(std::vector<double>& ener, std::vector<float>& force, std::vector<float>& virial,
                std::vector<float>& atom_energy, std::vector<float>& atom_virial, const std::vector<float>& coord,
                const std::vector<int>& atype, const std::vector<float>& box, const std::vector<float>& fparam,
                const std::vector<float>& aparam, const bool atomic) override {
    std::vector<double> f, v, ae, av;
    frames(ener, f, v, ae, av, to_double(coord), atype, to_double(box), fparam.size() + aparam.size(), atomic);
    from_double(force, f);
    from_double(virial, v);
    if (atomic) {
      from_double(atom_energy, ae);
      from_double(atom_virial, av);
    }
  }

  // ---- one frame with ghosts and the host's neighbour list
  void computew(std::vector<double>& ener, std::vector<double>& force, std::vector<double>& virial,
                std::vector<double>& atom_energy, std::vector<double>& atom_virial, const std::vector<double>& coord,
                const std::vector<int>& atype, const std::vector<double>& box, const int nghost,
                const deepmd::InputNlist& inlist, const int& ago, const std::vector<double>& fparam,
                const std::vector<double>& aparam, const bool atomic) override {
    (void)box;
    with_list(ener, force, virial, atom_energy, atom_virial, coord, atype, nghost, inlist, ago,
              fparam.size() + aparam.size(), atomic);
  }
  void computew(std::vector<double>& ener, std::vector<float>& force, std::vector<float>& virial,
                std::vector<float>& atom_energy, std::vector<float>& atom_virial, const std::vector<float>& coord,
                const std::vector<int>& atype, const std::vector<float>& box, const int nghost,
                const deepmd::InputNlist& inlist, const int& ago, const std::vector<float>& fparam,
                const std::vector<float>& aparam, const bool atomic) override {
    (void)box;
    std::vector<double> f, v, ae, av;
    with_list(ener, f, v, ae, av, to_double(coord), atype, nghost, inlist, ago, fparam.size() + aparam.size(),
              atomic);
    from_double(force, f);
    from_double(virial, v);
    if (atomic) {
      from_double(atom_energy, ae);
      from_double(atom_virial, av);
    }
  }

  // ---- frames with their own type vectors: one frame at a time
  void computew_mixed_type(std::vector<double>& ener, std::vector<double>& force, std::vector<double>& virial,
                           std::vector<double>& atom_energy, std::vector<double>& atom_virial, const int& nframes,
                           const std::vector<double>& coord, const std::vector<int>& atype,
                           const std::vector<double>& box, const std::vector<double>& fparam,
                           const std::vector<double>& aparam, const bool atomic) override {
    mixed(ener, force, virial, atom_energy, atom_virial, nframes, coord, atype, box, fparam.size() + aparam.size(),
          atomic);
  }
  void computew_mixed_type(std::vector<double>& ener, std::vector<float>& force, std::vector<float>& virial,
                           std::vector<float>& atom_energy, std::vector<float>& atom_virial, const int& nframes,
                           const std::vector<float>& coord, const std::vector<int>& atype,
                           const std::vector<float>& box, const std::vector<float>& fparam,
                           const std::vector<float>& aparam, const bool atomic) override {
    std::vector<double> f, v, ae, av;
    mixed(ener, f, v, ae, av, nframes, to_double(coord), atype, to_double(box), fparam.size() + aparam.size(),
          atomic);
    from_double(force, f);
    from_double(virial, v);
    if (atomic) {
      from_double(atom_energy, ae);
      from_double(atom_virial, av);
    }
  }

  // ---- graph inputs of message-passing models
  void compute_edges_gpu(double*, double*, double*, const double*, const int*, const int*, const double*, const int,
                         const int) override {
    raise("GB300 backend: se_e2_a models take no edge inputs");
  }
  void compute_edges_gpu(double*, double*, double*, const double*, const int*, const int*, const double*, const int,
                         const int, const std::vector<double>&, const std::vector<double>&, const int,
                         const deepmd::InputNlist*) override {
    raise("GB300 backend: se_e2_a models take no edge inputs");
  }
  void compute_edges_gpu(double*, double*, double*, const double*, const int*, const int*, const float*, const int,
                         const int, const std::vector<double>&, const std::vector<double>&, const int,
                         const deepmd::InputNlist*) override {
    raise("GB300 backend: se_e2_a models take no edge inputs");
  }
  void compute_canonical_graph_gpu(double*, double*, double*, const std::int64_t*, const std::int64_t*, const float*,
                                   const std::int64_t*, const std::int64_t*, const std::int64_t*, const int, const int,
                                   const std::int64_t) override {
    raise("GB300 backend: se_e2_a models take no graph inputs");
  }
  bool supports_device_edge_inference() const override { return false; }
  bool uses_fp32_edge_vectors() const override { return false; }
  bool uses_canonical_graph_inference() const override { return false; }

 private:
  void no_params(size_t n) const {
    if (n) raise("GB300 backend: the model has no frame or atomic parameters");
  }

  void frames(std::vector<double>& ener, std::vector<double>& force, std::vector<double>& virial,
              std::vector<double>& atom_energy, std::vector<double>& atom_virial, const std::vector<double>& coord,
              const std::vector<int>& atype, const std::vector<double>& box, size_t nparams, bool atomic) {
    no_params(nparams);
    const int natoms = (int)atype.size();
    if (natoms == 0 || coord.size() % (3 * (size_t)natoms)) raise("GB300 backend: coord and atype sizes disagree");
    const int nframes = (int)(coord.size() / (3 * (size_t)natoms));
    if (!box.empty() && box.size() != 9 * (size_t)nframes) raise("GB300 backend: box must hold 9 values per frame");
    ener.resize(nframes);
    force.resize(coord.size());
    virial.resize(9 * (size_t)nframes);
    if (atomic) {
      atom_energy.resize((size_t)nframes * natoms);
      atom_virial.resize((size_t)nframes * natoms * 9);
    }
    cudaSetDevice(device_);
    check(dpgb_deeppot_compute(dp_, nframes, natoms, coord.data(), atype.data(), box.empty() ? nullptr : box.data(),
                               ener.data(), force.data(), virial.data(), atomic ? atom_energy.data() : nullptr,
                               atomic ? atom_virial.data() : nullptr),
          dp_);
  }

  void with_list(std::vector<double>& ener, std::vector<double>& force, std::vector<double>& virial,
                 std::vector<double>& atom_energy, std::vector<double>& atom_virial, const std::vector<double>& coord,
                 const std::vector<int>& atype, int nghost, const deepmd::InputNlist& inlist, int ago,
                 size_t nparams, bool atomic) {
    no_params(nparams);
    const int nall = (int)atype.size();
    if (coord.size() != 3 * (size_t)nall) raise("GB300 backend: coord and atype sizes disagree");
    ener.resize(1);
    force.resize(3 * (size_t)nall);
    virial.resize(9);
    if (atomic) {
      atom_energy.resize(nall);
      atom_virial.resize(9 * (size_t)nall);
    }
    cudaSetDevice(device_);
    // ago > 0: the library keeps the list of the last call with ago == 0
    const bool fresh = ago == 0;
    check(dpgb_deeppot_compute_nlist(dp_, nall, nghost, coord.data(), atype.data(), nullptr,
                                     fresh ? inlist.inum : 0, fresh ? inlist.ilist : nullptr,
                                     fresh ? inlist.numneigh : nullptr,
                                     fresh ? const_cast<const int* const*>(inlist.firstneigh) : nullptr, ago,
                                     ener.data(), force.data(), virial.data(), atomic ? atom_energy.data() : nullptr,
                                     atomic ? atom_virial.data() : nullptr),
          dp_);
  }

  void mixed(std::vector<double>& ener, std::vector<double>& force, std::vector<double>& virial,
             std::vector<double>& atom_energy, std::vector<double>& atom_virial, int nframes,
             const std::vector<double>& coord, const std::vector<int>& atype, const std::vector<double>& box,
             size_t nparams, bool atomic) {
    no_params(nparams);
    if (nframes <= 0 || atype.size() % (size_t)nframes) raise("GB300 backend: atype is not nframes x natoms");
    const size_t natoms = atype.size() / nframes;
    if (coord.size() != 3 * natoms * nframes) raise("GB300 backend: coord is not nframes x natoms x 3");
    ener.assign(nframes, 0.0);
    force.assign(coord.size(), 0.0);
    virial.assign(9 * (size_t)nframes, 0.0);
    if (atomic) {
      atom_energy.assign(natoms * nframes, 0.0);
      atom_virial.assign(9 * natoms * nframes, 0.0);
    }
    for (int f = 0; f < nframes; ++f) {
      std::vector<double> e1, f1, v1, ae1, av1;
      const std::vector<double> c1(coord.begin() + 3 * natoms * f, coord.begin() + 3 * natoms * (f + 1));
      const std::vector<int> t1(atype.begin() + natoms * f, atype.begin() + natoms * (f + 1));
      const std::vector<double> b1 = box.empty() ? std::vector<double>()
                                                 : std::vector<double>(box.begin() + 9 * f, box.begin() + 9 * (f + 1));
      frames(e1, f1, v1, ae1, av1, c1, t1, b1, 0, atomic);
      ener[f] = e1[0];
      std::copy(f1.begin(), f1.end(), force.begin() + 3 * natoms * f);
      std::copy(v1.begin(), v1.end(), virial.begin() + 9 * f);
      if (atomic) {
        std::copy(ae1.begin(), ae1.end(), atom_energy.begin() + natoms * f);
        std::copy(av1.begin(), av1.end(), atom_virial.begin() + 9 * natoms * f);
      }
    }
  }

  dpgb_deeppot* dp_ = nullptr;
  int device_ = 0;
  double rcut_ = 0.0;
  int ntypes_ = 0;
  std::string type_map_;
};

char* copy_message(const std::string& m) {
  char* s = static_cast<char*>(std::malloc(m.size() + 1));
  if (s) std::memcpy(s, m.c_str(), m.size() + 1);
  return s;
}

}  // namespace

extern "C" {

__attribute__((visibility("default"))) void* deepmd_create_deeppot_backend_v1(const char* model, int gpu_rank,
                                                                              const char* file_content,
                                                                              std::size_t size,
                                                                              char** error_message) {
  if (error_message) *error_message = nullptr;
  try {
    auto* b = new DeepPotGB300();
    try {
      b->init(model ? model : "", gpu_rank, std::string(file_content ? file_content : "", file_content ? size : 0));
    } catch (...) {
      delete b;
      throw;
    }
    return static_cast<deepmd::DeepPotBackend*>(b);
  } catch (const std::exception& e) {
    if (error_message) *error_message = copy_message(e.what());
  } catch (...) {
    if (error_message) *error_message = copy_message("GB300 backend: unknown error");
  }
  return nullptr;
}

__attribute__((visibility("default"))) void deepmd_delete_deeppot_backend_v1(void* backend) {
  delete static_cast<deepmd::DeepPotBackend*>(backend);
}

__attribute__((visibility("default"))) void deepmd_free_backend_error_v1(char* error_message) {
  std::free(error_message);
}

}  // extern "C"
