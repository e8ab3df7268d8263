// Test host (not shipped): loads a DeepPot backend plugin the way a
// reference host does (dlopen + the three C symbols, BackendPlugin.cc) and
// drives it through deepmd::DeepPotBackend's virtual methods.
//   host <plugin.so> <model.pth> <jobs.bin> <out.bin>
// jobs.bin: int32 njobs, then per job an int32 kind and its inputs:
//   0 frames, FP64:  nframes natoms | coord f64[nf*na*3] | atype i32[na] | hasbox | box f64[nf*9]
//   1 frames, FP32:  the same, coordinates and box converted to float
//   2 neighbour list, FP64: nall nghost | coord f64[nall*3] | atype i32[nall] | inum |
//                    ilist i32[inum] | numneigh i32[inum] | neighbours i32[sum numneigh] | ago
//   3 mixed types, FP64: nframes natoms | coord | atype i32[nf*na] | hasbox | box
// out.bin: per job five arrays (energy, force, virial, atom energy, atom
// virial), each as int64 length + f64 values.  A creation failure prints
// the plugin's message and exits 3.
#include <dlfcn.h>

#include <cstdint>
#include <cstdio>
#include <fstream>
#include <string>
#include <vector>

#include "deepmd_backend_abi.h"

using VD = std::vector<double>;

template <typename T>
std::vector<T> rd(std::ifstream& f, size_t n) {
  std::vector<T> v(n);
  f.read(reinterpret_cast<char*>(v.data()), sizeof(T) * n);
  return v;
}
int rdi(std::ifstream& f) { return rd<int32_t>(f, 1)[0]; }

template <typename V>
void put(std::ofstream& o, const std::vector<V>& v) {
  const int64_t n = (int64_t)v.size();
  o.write(reinterpret_cast<const char*>(&n), sizeof(n));
  for (auto x : v) {
    const double d = (double)x;
    o.write(reinterpret_cast<const char*>(&d), sizeof(d));
  }
}

int main(int argc, char** argv) {
  if (argc != 5) return 2;
  void* h = dlopen(argv[1], RTLD_NOW | RTLD_LOCAL);
  if (!h) {
    std::fprintf(stderr, "dlopen: %s\n", dlerror());
    return 2;
  }
  auto create = reinterpret_cast<void* (*)(const char*, int, const char*, std::size_t, char**)>(
      dlsym(h, "deepmd_create_deeppot_backend_v1"));
  auto destroy = reinterpret_cast<void (*)(void*)>(dlsym(h, "deepmd_delete_deeppot_backend_v1"));
  auto free_err = reinterpret_cast<void (*)(char*)>(dlsym(h, "deepmd_free_backend_error_v1"));
  if (!create || !destroy || !free_err) return 2;
  char* err = nullptr;
  void* raw = create(argv[2], 0, "", 0, &err);
  if (!raw) {
    std::printf("create failed: %s\n", err ? err : "(no message)");
    free_err(err);
    return 3;
  }
  auto* dp = static_cast<deepmd::DeepPotBackend*>(raw);
  std::string tm;
  dp->get_type_map(tm);
  std::printf("cutoff %g ntypes %d type_map %s fparam %d aparam %d\n", dp->cutoff(), dp->numb_types(), tm.c_str(),
              dp->dim_fparam(), dp->dim_aparam());
  std::ifstream in(argv[3], std::ios::binary);
  std::ofstream out(argv[4], std::ios::binary);
  const int njobs = rdi(in);
  int rc = 0;
  for (int j = 0; j < njobs; ++j) {
    const int kind = rdi(in);
    VD e, f, v, ae, av;
    try {
      if (kind == 0 || kind == 1 || kind == 3) {
        const int nf = rdi(in), na = rdi(in);
        const VD c = rd<double>(in, (size_t)nf * na * 3);
        const std::vector<int> t = rd<int32_t>(in, (size_t)(kind == 3 ? nf : 1) * na);
        const int hasbox = rdi(in);
        const VD b = hasbox ? rd<double>(in, (size_t)nf * 9) : VD();
        if (kind == 0) {
          dp->computew(e, f, v, ae, av, c, t, b, VD(), VD(), true);
        } else if (kind == 3) {
          dp->computew_mixed_type(e, f, v, ae, av, nf, c, t, b, VD(), VD(), true);
        } else {
          std::vector<float> cf(c.begin(), c.end()), bf(b.begin(), b.end()), ff, vf, aef, avf;
          dp->computew(e, ff, vf, aef, avf, cf, t, bf, std::vector<float>(), std::vector<float>(), true);
          f.assign(ff.begin(), ff.end());
          v.assign(vf.begin(), vf.end());
          ae.assign(aef.begin(), aef.end());
          av.assign(avf.begin(), avf.end());
        }
      } else if (kind == 2) {
        const int nall = rdi(in), nghost = rdi(in);
        const VD c = rd<double>(in, (size_t)nall * 3);
        const std::vector<int> t = rd<int32_t>(in, nall);
        const int inum = rdi(in);
        std::vector<int> ilist = rd<int32_t>(in, inum), numneigh = rd<int32_t>(in, inum);
        std::vector<std::vector<int>> rows(inum);
        std::vector<int*> first(inum);
        for (int i = 0; i < inum; ++i) {
          rows[i] = rd<int32_t>(in, numneigh[i]);
          first[i] = rows[i].data();
        }
        const int ago = rdi(in);
        deepmd::InputNlist nl(inum, ilist.data(), numneigh.data(), first.data());
        dp->computew(e, f, v, ae, av, c, t, VD(), nghost, nl, ago, VD(), VD(), true);
      } else {
        return 2;
      }
    } catch (const deepmd::deepmd_exception& ex) {  // the type a reference host catches
      std::printf("job %d: %s\n", j, ex.what());
      rc = 4;
    }
    put(out, e);
    put(out, f);
    put(out, v);
    put(out, ae);
    put(out, av);
  }
  destroy(raw);
  return rc;
}
