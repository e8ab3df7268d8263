// Op-level environment matrix and force / virial products.
//
// prod_env_mat_a: the reference C++ semantics (source/lib/src/env_mat.cc:
// 123-223, prod_env_mat.cc:14-132): the switching radii are the float values
// the reference passes (`const float& rmin/rmax`), padding slots hold
// (0 - avg)/std, virtual centres are zero.
// env_mat_pt: the PyTorch semantics of deepmd/pt/model/descriptor/env_mat.py.
// prod_force_a / prod_virial_a: per-pair products first, then a gather through
// the sorted transpose of the list (no atomics, bitwise reproducible).
#include <vector>

#include "nlist.cuh"

namespace dpgb {
namespace {

// the reference switch takes float radii: the width rmax - rmin is a float
// subtraction (source/lib/include/switcher.h spline5_switch)
__device__ __forceinline__ void switch5(double x, float rmin, float rmax, double& vv, double& dd) {
  if (x < rmin) {
    dd = 0.0;
    vv = 1.0;
  } else if (x < rmax) {
    const float w = __fsub_rn(rmax, rmin);
    const double uu = (x - rmin) / w;
    const double du = 1.0 / w;
    vv = uu * uu * uu * (-6.0 * uu * uu + 15.0 * uu - 10.0) + 1.0;
    dd = (3.0 * uu * uu * (-6.0 * uu * uu + 15.0 * uu - 10.0) + uu * uu * uu * (-12.0 * uu + 15.0)) * du;
  } else {
    dd = 0.0;
    vv = 0.0;
  }
}

// one thread per (row, slot)
__global__ void env_mat_a_kernel(double* __restrict__ em, double* __restrict__ em_deriv,
                                 double* __restrict__ rij, const int* __restrict__ nlist,
                                 const double* __restrict__ coord, const int* __restrict__ atype,
                                 const double* __restrict__ avg, const double* __restrict__ std,
                                 int nloc, int nnei, float rmin, float rmax) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= (long long)nloc * nnei) return;
  const int i = (int)(q / nnei), jj = (int)(q % nnei);
  const int ti = atype[i];
  const int j = nlist[q];  // written by the formatter: -1 or a checked index < nall
  double e4[4] = {0, 0, 0, 0}, dv[12], d[3] = {0, 0, 0};
#pragma unroll
  for (int k = 0; k < 12; ++k) dv[k] = 0.0;
  if (j >= 0) {
#pragma unroll
    for (int k = 0; k < 3; ++k) d[k] = coord[3 * j + k] - coord[3 * i + k];
    const double nr2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    const double inr = 1.0 / sqrt(nr2);
    const double nr = nr2 * inr;
    const double inr2 = inr * inr, inr4 = inr2 * inr2, inr3 = inr4 * nr;
    double sw, dsw;
    switch5(nr, rmin, rmax, sw, dsw);
    const double v0 = 1.0 / nr;
    const double v[3] = {d[0] / nr2, d[1] / nr2, d[2] / nr2};
#pragma unroll
    for (int k = 0; k < 3; ++k) dv[k] = d[k] * inr3 * sw - v0 * dsw * d[k] * inr;
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int k = 0; k < 3; ++k)
        dv[3 + 3 * c + k] = (2.0 * d[c] * d[k] * inr4 - (c == k ? inr2 : 0.0)) * sw - v[c] * dsw * d[k] * inr;
    e4[0] = v0 * sw;
#pragma unroll
    for (int c = 0; c < 3; ++c) e4[1 + c] = v[c] * sw;
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) rij[3 * q + k] = d[k];
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    const size_t a = ((size_t)(ti >= 0 ? ti : 0) * nnei + jj) * 4 + c;
    em[4 * q + c] = ti >= 0 ? (e4[c] - avg[a]) / std[a] : 0.0;
#pragma unroll
    for (int k = 0; k < 3; ++k) em_deriv[12 * q + 3 * c + k] = ti >= 0 ? dv[3 * c + k] / std[a] : 0.0;
  }
}

// PyTorch env_mat: t0 = 1/len, t1 = diff/len^2, times the switch, masked,
// then (env - avg[t]) / std[t]  (env_mat.py:18-55,115-118)
__global__ void env_mat_pt_kernel(double* __restrict__ em, double* __restrict__ diff,
                                  double* __restrict__ swo, const int* __restrict__ nlist,
                                  const double* __restrict__ coord, const int* __restrict__ atype,
                                  const double* __restrict__ avg, const double* __restrict__ std,
                                  int nf, int nloc, int nall, int nnei, double rmin, double rmax) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= (long long)nf * nloc * nnei) return;
  const long long row = q / nnei;
  const int jj = (int)(q % nnei);
  const int f = (int)(row / nloc), i = (int)(row % nloc);
  const double* cf = coord + (size_t)f * nall * 3;
  const int ti = atype[(size_t)f * nall + i];
  int j = nlist[q];
  if (j >= nall) j = -1;  // out-of-range entries are treated as padding, never dereferenced
  double d[3] = {0, 0, 0}, e4[4] = {0, 0, 0, 0}, w = 0.0;
  if (j >= 0) {
#pragma unroll
    for (int k = 0; k < 3; ++k) d[k] = cf[3 * j + k] - cf[3 * i + k];
    const double len = sqrt(fma(d[2], d[2], fma(d[1], d[1], d[0] * d[0])));
    const double xx = fmin(fmax(len, rmin), rmax);
    const double uu = (xx - rmin) / (rmax - rmin);
    const double uu2 = uu * uu;
    w = uu2 * uu * (-6.0 * uu2 + 15.0 * uu - 10.0) + 1.0;
    const double l2 = len * len;
    e4[0] = 1.0 / len * w;
#pragma unroll
    for (int k = 0; k < 3; ++k) e4[1 + k] = d[k] / l2 * w;
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) diff[3 * q + k] = d[k];
  swo[q] = w;
  const int tt = ti >= 0 ? ti : 0;
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    const size_t a = ((size_t)tt * nnei + jj) * 4 + c;
    em[4 * q + c] = (e4[c] - avg[a]) / std[a];
  }
}

// per-pair force p = sum_{a in slot} net_deriv[a] * env_deriv[a, :]
__global__ void pair_force_kernel(double* __restrict__ pf, const double* __restrict__ nd,
                                  const double* __restrict__ ed, long long npair) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npair) return;
  double f[3] = {0, 0, 0};
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    const double n = nd[4 * p + a];
#pragma unroll
    for (int k = 0; k < 3; ++k) f[k] += n * ed[(4 * p + a) * 3 + k];
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) pf[3 * p + k] = f[k];
}

// force[f, j] = -sum_slots pf[row j] (centre, j < nloc) + sum_{pairs -> j} pf
__global__ void force_gather_kernel(double* __restrict__ force, const double* __restrict__ pf,
                                    Transpose tr, int nloc, int nall, int nnei, int nframes) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= (long long)nframes * nall) return;
  const int f = (int)(q / nall), j = (int)(q % nall);
  double acc[3] = {0, 0, 0};
  if (j < nloc) {
    const double* row = pf + ((size_t)f * nloc + j) * nnei * 3;
    for (int s = 0; s < nnei; ++s)
#pragma unroll
      for (int k = 0; k < 3; ++k) acc[k] -= row[3 * s + k];
  }
  for (int t = tr.offsets[q]; t < tr.offsets[q + 1]; ++t) {
    const int p = tr.pairs[t];
#pragma unroll
    for (int k = 0; k < 3; ++k) acc[k] += pf[3 * (size_t)p + k];
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) force[3 * q + k] = acc[k];
}

__global__ void frame_keys_kernel(int* __restrict__ keys, const int* __restrict__ nlist, long long npair,
                                  long long per_frame, int nall) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npair) return;
  const int j = nlist[p];
  keys[p] = (j < 0 || j >= nall) ? -1 : (int)(j + (p / per_frame) * nall);
}

// per-pair virial pv[9] = sum_a nd[a] * rij[d1] * ed[a][d0]
__global__ void pair_virial_kernel(double* __restrict__ pv, const double* __restrict__ nd,
                                   const double* __restrict__ ed, const double* __restrict__ rij,
                                   const int* __restrict__ nlist, long long npair) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npair) return;
  double v[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) v[k] = 0.0;
  if (nlist[p] >= 0) {
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      const double n = nd[4 * p + a];
#pragma unroll
      for (int d0 = 0; d0 < 3; ++d0)
#pragma unroll
        for (int d1 = 0; d1 < 3; ++d1) v[d0 * 3 + d1] += n * rij[3 * p + d1] * ed[(4 * p + a) * 3 + d0];
    }
  }
#pragma unroll
  for (int k = 0; k < 9; ++k) pv[9 * p + k] = v[k];
}

__global__ void atom_virial_gather_kernel(double* __restrict__ av, const double* __restrict__ pv,
                                          Transpose tr, int nall) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nall) return;
  double acc[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) acc[k] = 0.0;
  for (int t = tr.offsets[j]; t < tr.offsets[j + 1]; ++t) {
    const int p = tr.pairs[t];
#pragma unroll
    for (int k = 0; k < 9; ++k) acc[k] += pv[9 * (size_t)p + k];
  }
#pragma unroll
  for (int k = 0; k < 9; ++k) av[9 * (size_t)j + k] = acc[k];
}

// deterministic column sums of a [n, w] FP64 array: one block per column
__global__ void column_sum_kernel(double* __restrict__ out, const double* __restrict__ in, int n, int w) {
  __shared__ double s[256];
  const int c = blockIdx.x;
  double acc = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) acc += in[(size_t)i * w + c];
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[c] = s[0];
}

__global__ void force_grad_kernel(double* __restrict__ gn, const double* __restrict__ grad,
                                  const double* __restrict__ ed, const int* __restrict__ nlist,
                                  int nloc, int nnei, long long total) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;  // (row, a)
  if (q >= total) return;
  const long long row = q / (4 * nnei);
  const int a = (int)(q % (4 * nnei));
  const int slot = a / 4;
  const int f = (int)(row / nloc);
  const double* e = ed + 3 * q;
  double v = 0.0;
#pragma unroll
  for (int k = 0; k < 3; ++k) v -= grad[3 * row + k] * e[k];
  int j = nlist[row * nnei + slot];
  if (j >= nloc) j = j % nloc;
  if (j >= 0) {
#pragma unroll
    for (int k = 0; k < 3; ++k) v += grad[((size_t)f * nloc + j) * 3 + k] * e[k];
  }
  gn[q] = v;
}

__global__ void virial_grad_kernel(double* __restrict__ gn, const double* __restrict__ grad,
                                   const double* __restrict__ ed, const double* __restrict__ rij,
                                   const int* __restrict__ nlist, int nnei, long long total) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= total) return;
  const long long pair = q / 4;
  double v = 0.0;
  if (nlist[pair] >= 0) {
#pragma unroll
    for (int d0 = 0; d0 < 3; ++d0)
#pragma unroll
      for (int d1 = 0; d1 < 3; ++d1) v += grad[d0 * 3 + d1] * rij[3 * pair + d1] * ed[3 * q + d0];
  }
  gn[q] = v;
}

}  // namespace
}  // namespace dpgb

using namespace dpgb;

extern "C" {

int dpgb_prod_env_mat_a_f64(double* em, double* em_deriv, double* rij, int* nlist,
                            const double* coord, const int* atype, const int* rows,
                            const int* counts, int max_nbor, const double* avg, const double* std,
                            int nloc, int nall, double rcut, double rcut_smth, const int* sel_host,
                            int ntypes, void* stream) {
  clear_error();
  SelInfo sel;
  DPGB_TRY(sel_from_host(sel_host, ntypes, sel));
  if (nloc < 0 || nall < nloc) return fail(DPGB_EINVAL, "prod_env_mat_a: bad sizes");
  if (nloc == 0) return DPGB_OK;
  if (!em || !em_deriv || !rij || !nlist || !coord || !atype || !avg || !std || !counts)
    return fail(DPGB_EINVAL, "prod_env_mat_a: NULL pointer");
  int ovf = 0;
  DPGB_TRY(dpgb_format_nlist_a(nlist, coord, atype, rows, counts, max_nbor, nloc, nall, rcut, sel_host,
                               ntypes, &ovf, stream));
  const long long tot = (long long)nloc * sel.nnei;
  if (tot == 0) return DPGB_OK;
  // the reference evaluates the switch with float radii (env_mat.cc:132-133)
  env_mat_a_kernel<<<ceil_div(tot, 128), 128, 0, as_stream(stream)>>>(
      em, em_deriv, rij, nlist, coord, atype, avg, std, nloc, sel.nnei, (float)rcut_smth, (float)rcut);
  return check_launch("prod_env_mat_a");
}

int dpgb_env_mat_pt_f64(double* em, double* diff, double* sw, const double* coord,
                        const int* atype, const int* nlist, const double* avg, const double* std,
                        int nf, int nloc, int nall, int nnei, double rcut, double rcut_smth,
                        void* stream) {
  clear_error();
  if (nf < 0 || nloc < 0 || nall < nloc || nnei < 0) return fail(DPGB_EINVAL, "env_mat_pt: bad sizes");
  if (!(rcut_smth < rcut)) return fail(DPGB_EINVAL, "rmin should be less than rmax.");
  const long long tot = (long long)nf * nloc * nnei;
  if (tot == 0) return DPGB_OK;
  env_mat_pt_kernel<<<ceil_div(tot, 128), 128, 0, as_stream(stream)>>>(
      em, diff, sw, nlist, coord, atype, avg, std, nf, nloc, nall, nnei, rcut_smth, rcut);
  return check_launch("env_mat_pt");
}

int dpgb_prod_force_a_f64(double* force, const double* nd, const double* ed, const int* nlist,
                          int nloc, int nall, int nnei, int nframes, void* stream) {
  clear_error();
  if (nloc < 0 || nall < nloc || nnei < 0 || nframes < 1) return fail(DPGB_EINVAL, "prod_force_a: bad sizes");
  cudaStream_t st = as_stream(stream);
  const long long npair = (long long)nframes * nloc * nnei;
  const long long nkeys = (long long)nframes * nall;
  if (nkeys == 0) return DPGB_OK;
  if (nkeys >= (1LL << 31) || npair >= (1LL << 31)) return fail(DPGB_EINVAL, "prod_force_a: too large");
  DeviceBuffer ws;
  const size_t pf_bytes = sizeof(double) * 3 * (size_t)npair;
  const size_t key_bytes = sizeof(int) * (size_t)npair;
  const size_t tr_bytes = transpose_workspace(npair, (int)nkeys);
  DPGB_TRY(ws.alloc(pf_bytes + key_bytes + tr_bytes + sizeof(int) * kStatusSlots + 64));
  double* pf = ws.as<double>();
  int* keys = reinterpret_cast<int*>(reinterpret_cast<char*>(pf) + pf_bytes);
  int* status = keys + npair;
  void* trw = status + kStatusSlots;
  DPGB_CUDA(cudaMemsetAsync(status, 0, sizeof(int) * kStatusSlots, st));
  if (npair > 0) {
    pair_force_kernel<<<ceil_div(npair, 256), 256, 0, st>>>(pf, nd, ed, npair);
    DPGB_TRY(check_launch("pair_force"));
    frame_keys_kernel<<<ceil_div(npair, 256), 256, 0, st>>>(keys, nlist, npair, (long long)nloc * nnei, nall);
    DPGB_TRY(check_launch("frame_keys"));
  }
  Transpose tr;
  DPGB_TRY(launch_transpose(tr, keys, npair, (int)nkeys, 0, trw, status, st));
  force_gather_kernel<<<ceil_div(nkeys, 256), 256, 0, st>>>(force, pf, tr, nloc, nall, nnei, nframes);
  DPGB_TRY(check_launch("force_gather"));
  int h[kStatusSlots];
  DPGB_TRY(read_status(status, st, h));  // also keeps the workspace alive until done
  if (h[kStatusOverflow] > 0) return fail(DPGB_EOVERFLOW, "prod_force_a: an atom appears in more than 2048 rows");
  return DPGB_OK;
}

int dpgb_prod_virial_a_f64(double* virial, double* atom_virial, const double* nd, const double* ed,
                           const double* rij, const int* nlist, int nloc, int nall, int nnei,
                           void* stream) {
  clear_error();
  if (nloc < 0 || nall < nloc || nnei < 0) return fail(DPGB_EINVAL, "prod_virial_a: bad sizes");
  cudaStream_t st = as_stream(stream);
  const long long npair = (long long)nloc * nnei;
  DeviceBuffer ws;
  const size_t pv_bytes = sizeof(double) * 9 * (size_t)npair;
  const size_t tr_bytes = transpose_workspace(npair, nall);
  DPGB_TRY(ws.alloc(pv_bytes + tr_bytes + sizeof(int) * kStatusSlots + 64));
  double* pv = ws.as<double>();
  int* status = reinterpret_cast<int*>(reinterpret_cast<char*>(pv) + pv_bytes);
  void* trw = status + kStatusSlots;
  DPGB_CUDA(cudaMemsetAsync(status, 0, sizeof(int) * kStatusSlots, st));
  if (npair > 0) {
    pair_virial_kernel<<<ceil_div(npair, 256), 256, 0, st>>>(pv, nd, ed, rij, nlist, npair);
    DPGB_TRY(check_launch("pair_virial"));
  }
  Transpose tr;
  DPGB_TRY(launch_transpose(tr, nlist, npair, nall, 0, trw, status, st));
  if (nall > 0) {
    atom_virial_gather_kernel<<<ceil_div(nall, 256), 256, 0, st>>>(atom_virial, pv, tr, nall);
    DPGB_TRY(check_launch("atom_virial_gather"));
    column_sum_kernel<<<9, 256, 0, st>>>(virial, atom_virial, nall, 9);
    DPGB_TRY(check_launch("virial_sum"));
  } else {
    DPGB_CUDA(cudaMemsetAsync(virial, 0, sizeof(double) * 9, st));
  }
  int h[kStatusSlots];
  DPGB_TRY(read_status(status, st, h));
  if (h[kStatusOverflow] > 0) return fail(DPGB_EOVERFLOW, "prod_virial_a: an atom appears in more than 2048 rows");
  return DPGB_OK;
}

int dpgb_prod_force_grad_a_f64(double* gn, const double* grad, const double* ed, const int* nlist,
                               int nloc, int nnei, int nframes, void* stream) {
  clear_error();
  if (nloc < 0 || nnei < 0 || nframes < 1) return fail(DPGB_EINVAL, "prod_force_grad_a: bad sizes");
  const long long total = (long long)nframes * nloc * nnei * 4;
  if (total == 0) return DPGB_OK;
  force_grad_kernel<<<ceil_div(total, 256), 256, 0, as_stream(stream)>>>(gn, grad, ed, nlist, nloc, nnei, total);
  return check_launch("prod_force_grad_a");
}

int dpgb_prod_virial_grad_a_f64(double* gn, const double* grad, const double* ed, const double* rij,
                                const int* nlist, int nloc, int nnei, void* stream) {
  clear_error();
  if (nloc < 0 || nnei < 0) return fail(DPGB_EINVAL, "prod_virial_grad_a: bad sizes");
  const long long total = (long long)nloc * nnei * 4;
  if (total == 0) return DPGB_OK;
  virial_grad_kernel<<<ceil_div(total, 256), 256, 0, as_stream(stream)>>>(gn, grad, ed, rij, nlist, nnei, total);
  return check_launch("prod_virial_grad_a");
}

}  // extern "C"
