// Compression tables of se_e2_a embedding nets, built on the GPU: the
// fifth-order piecewise polynomial of deepmd/utils/tabulate.py:275-370
// (_build_lower) over the node grid of tabulate.py:67-148 (build), with the
// node values, first and second derivatives of the net computed analytically
// (deepmd/utils/tabulate_math.py:353-470 _make_data).
//
// Grid: x_i = lower + i*delta0 for i < n0 = ceil((upper - lower) / stride0),
// then upper + i*delta1 for i < n1 = ceil((extrapolate*upper - upper) /
// stride1), then extrapolate*upper — numpy.arange's fill, whose step is
// delta = (start + stride) - start.  Row r < nspline, neuron n, with h the
// row's stride (stride0 for the first int((upper - lower)/stride0) rows,
// stride1 after) and dv = v[r+1] - v[r], holds the quintic Hermite
// coefficients of the interval:
//   a0 = v0, a1 = d0, a2 = d2_0 / 2,
//   a3 = (20 dv - (8 d1 + 12 d0) h - (3 s0 - s1) h^2) / (2 h^3),
//   a4 = (-30 dv + (14 d1 + 16 d0) h + (3 s0 - 2 s1) h^2) / (2 h^4),
//   a5 = (12 dv - 6 (d1 + d0) h + (s1 - s0) h^2) / (2 h^5)
// (d = first, s = second derivative; 0/1 = left/right node).  As in the
// reference, a layer's timestep (idt) is not applied in the tabulated net.
#include <algorithm>
#include <cmath>

#include "common.cuh"

namespace dpgb {
namespace {

struct TabNet {
  int n_layer;
  int width[DPGB_MAX_LAYERS + 1];
  int woff[DPGB_MAX_LAYERS], boff[DPGB_MAX_LAYERS];
  int maxw;
};

struct TabGrid {
  double lower, upper, xmax, delta0, delta1;
  int n0, n1, nnode;
};

__device__ __forceinline__ double node_x(const TabGrid& g, int i) {
  if (i < g.n0) return g.lower + i * g.delta0;
  if (i < g.n0 + g.n1) return g.upper + (i - g.n0) * g.delta1;
  return g.xmax;
}

// one CTA per node: value, d/dx, d2/dx2 of every output neuron
__global__ void node_kernel(double* __restrict__ vdd, const double* __restrict__ W, TabNet net, TabGrid grid) {
  extern __shared__ double sm[];
  const int node = blockIdx.x, tid = threadIdx.x;
  double* a = sm;                  // [3][maxw] current layer: value, d1, d2
  double* b = sm + 3 * net.maxw;   // [3][maxw] next layer
  if (tid == 0) {
    a[0] = node_x(grid, node);
    a[net.maxw] = 1.0;
    a[2 * net.maxw] = 0.0;
  }
  __syncthreads();
  for (int l = 1; l <= net.n_layer; ++l) {
    const int nin = net.width[l - 1], nout = net.width[l];
    const double* Wm = W + net.woff[l - 1];
    const double* bias = W + net.boff[l - 1];
    for (int n = tid; n < nout; n += blockDim.x) {
      double z = bias[n], z1 = 0.0, z2 = 0.0;
      for (int k = 0; k < nin; ++k) {
        const double w = Wm[k * nout + n];
        z += a[k] * w;
        z1 += a[net.maxw + k] * w;
        z2 += a[2 * net.maxw + k] * w;
      }
      const double t = tanh(z), g1 = 1.0 - t * t;
      double y = t, y1 = g1 * z1, y2 = g1 * z2 - 2.0 * t * g1 * z1 * z1;
      if (nout == nin || nout == 2 * nin) {
        const int k = nout == nin ? n : n % nin;
        y += a[k];
        y1 += a[net.maxw + k];
        y2 += a[2 * net.maxw + k];
      }
      b[n] = y;
      b[net.maxw + n] = y1;
      b[2 * net.maxw + n] = y2;
    }
    __syncthreads();
    double* s = a;
    a = b;
    b = s;
  }
  const int ng = net.width[net.n_layer];
  for (int n = tid; n < ng; n += blockDim.x) {
    vdd[((size_t)0 * grid.nnode + node) * ng + n] = a[n];
    vdd[((size_t)1 * grid.nnode + node) * ng + n] = a[net.maxw + n];
    vdd[((size_t)2 * grid.nnode + node) * ng + n] = a[2 * net.maxw + n];
  }
}

__global__ void coeff_kernel(double* __restrict__ table, const double* __restrict__ vdd, int nnode, int ng,
                             int nspline, int nrow0, double stride0, double stride1) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= (long long)nspline * ng) return;
  const int r = (int)(q / ng), n = (int)(q - (long long)r * ng);
  const double h = r < nrow0 ? stride0 : stride1;
  const double* v = vdd;
  const double* d = vdd + (size_t)nnode * ng;
  const double* s = vdd + (size_t)2 * nnode * ng;
  const double v0 = v[(size_t)r * ng + n], v1 = v[(size_t)(r + 1) * ng + n];
  const double d0 = d[(size_t)r * ng + n], d1 = d[(size_t)(r + 1) * ng + n];
  const double s0 = s[(size_t)r * ng + n], s1 = s[(size_t)(r + 1) * ng + n];
  const double dv = v1 - v0;
  double* o = table + (size_t)r * 6 * ng + 6 * n;
  o[0] = v0;
  o[1] = d0;
  o[2] = 0.5 * s0;
  o[3] = (1.0 / (2.0 * h * h * h)) * (20.0 * dv - (8.0 * d1 + 12.0 * d0) * h - (3.0 * s0 - s1) * h * h);
  o[4] = (1.0 / (2.0 * h * h * h * h)) * (-30.0 * dv + (14.0 * d1 + 16.0 * d0) * h + (3.0 * s0 - 2.0 * s1) * h * h);
  o[5] = (1.0 / (2.0 * h * h * h * h * h)) * (12.0 * dv - 6.0 * (d1 + d0) * h + (s1 - s0) * h * h);
}

}  // namespace
}  // namespace dpgb

using namespace dpgb;

extern "C" {

int dpgb_se_a_table_rows(double lower, double upper, double extrapolate, double stride0, double stride1) {
  if (!(upper > lower) || !(stride0 > 0) || !(stride1 > 0) || !(extrapolate >= 1)) return -1;
  return (int)((upper - lower) / stride0 + (extrapolate * upper - upper) / stride1);
}

int dpgb_se_a_table_build_f64(double* table, const dpgb_se_a_block* b, const double* params, int net, double lower,
                              double upper, double extrapolate, double stride0, double stride1, void* stream) {
  clear_error();
  if (!table || !b || !params) return fail(DPGB_EINVAL, "table_build: NULL pointer");
  if (b->n_layer < 1 || b->n_layer > DPGB_MAX_LAYERS) return fail(DPGB_EINVAL, "table_build: bad n_layer");
  const int nnets = b->type_one_side ? b->ntypes : b->ntypes * b->ntypes;
  if (net < 0 || net >= nnets) return fail(DPGB_EINVAL, "table_build: net index out of range");
  const int nspline = dpgb_se_a_table_rows(lower, upper, extrapolate, stride0, stride1);
  if (nspline < 1) return fail(DPGB_EINVAL, "table_build: empty or invalid range");
  TabNet tn{};
  tn.n_layer = b->n_layer;
  tn.width[0] = 1;
  tn.maxw = 1;
  int off = 0;
  for (int l = 0; l < b->n_layer; ++l) {
    const int nin = l == 0 ? 1 : b->neuron[l - 1], nout = b->neuron[l];
    if (nout < 1 || nout > 1024) return fail(DPGB_EINVAL, "table_build: bad width");
    tn.width[l + 1] = nout;
    tn.maxw = std::max(tn.maxw, nout);
    tn.woff[l] = off;
    off += nin * nout;
    tn.boff[l] = off;
    off += nout;
    if (b->resnet_dt) off += nout;
  }
  const double* W = params + (size_t)net * off;
  TabGrid g{};
  g.lower = lower;
  g.upper = upper;
  g.xmax = extrapolate * upper;
  g.delta0 = (lower + stride0) - lower;
  g.delta1 = (upper + stride1) - upper;
  g.n0 = (int)std::ceil((upper - lower) / stride0);
  g.n1 = (int)std::ceil((extrapolate * upper - upper) / stride1);
  if (g.n1 < 0) g.n1 = 0;
  g.nnode = g.n0 + g.n1 + 1;
  if (g.nnode < nspline + 1) return fail(DPGB_EINVAL, "table_build: node grid shorter than the table");
  const int ng = tn.width[tn.n_layer];
  cudaStream_t st = as_stream(stream);
  DeviceBuffer vdd;
  DPGB_TRY(vdd.alloc(sizeof(double) * 3 * (size_t)g.nnode * ng));
  node_kernel<<<g.nnode, 128, sizeof(double) * 6 * tn.maxw, st>>>(vdd.as<double>(), W, tn, g);
  DPGB_TRY(check_launch("table_build_nodes"));
  const long long n = (long long)nspline * ng;
  coeff_kernel<<<ceil_div(n, 128), 128, 0, st>>>(table, vdd.as<double>(), g.nnode, ng, nspline,
                                                 (int)((upper - lower) / stride0), stride0, stride1);
  DPGB_TRY(check_launch("table_build_coeffs"));
  DPGB_CUDA(cudaStreamSynchronize(st));  // the node buffer is freed on return
  return DPGB_OK;
}

}  // extern "C"
