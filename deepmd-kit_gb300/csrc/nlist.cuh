// Neighbour-list building blocks shared by the op-level entry points and the
// DeepPot pipeline.
#pragma once

#include <vector>

#include "common.cuh"

namespace dpgb {

// kStatusTruncated: widest type section a strict list (SelInfo::strict) lacked
// kStatusExact: atoms whose list needed exact FP64 distances (FP32 ambiguous)
enum StatusExtra { kStatusDropped = 3, kStatusTruncated = 4, kStatusExact = 5 };

// Cell-list geometry of one frame (host-computed, passed by value).
struct CellGeom {
  double cell[9];     // rows are the cell vectors
  double rec[9];      // inverse of cell
  double origin[3];   // open boundary: lower corner of the atoms' bounding box
  double csize[3];    // open boundary: cell edge
  int ncell[3];       // cells per direction
  int reach[3];       // stencil half-width in cells
  int nbuff[3];       // periodic image range (reference nbuff)
  int nshift;
  int zero_shift;     // position of the (0,0,0) image
  int periodic;
  float eps;          // error bound of the staged FP32 distances (staged_eps)
};

struct SelInfo {
  int ntypes;
  int nnei;
  int sel[DPGB_MAX_TYPES];
  int sec[DPGB_MAX_TYPES + 1];
  // 1: a pair within the cutoff that finds no slot (beyond sum(sel) or its
  // type's sel) raises kStatusTruncated to its rank within its type + 1 (the
  // width its type would need) — for candidate lists, which must hold every
  // pair
  int strict;
  // 1: rows are flat candidate lists (every pair within the cutoff, at its
  // rank over all types or in search order; no per-type sections)
  int flat;
};

// Sorted transpose of a list: for key k, pairs[offsets[k] .. offsets[k+1])
// are the pair ids p (ascending) with keys[p] (mod `mod`) == k.
struct Transpose {
  int* offsets = nullptr;
  int* pairs = nullptr;
  int nkeys = 0;
};

// cell, inverse cell and face distances of a periodic box
int box_geom(const double* box, CellGeom& g);
// periodic cell list + image table for the reference's image order
int periodic_geom(const double* box, double rcut, int nshift, const int* shift_idx, CellGeom& g,
                  std::vector<int>& shift_pos);
// open boundary: bounding box of host coordinates
int open_geom(const double* coord_host, int n, double rcut, CellGeom& g);
void shift_vectors(const CellGeom& g, const int* shift_idx, int nshift, std::vector<double>& out);

// status (may be NULL): flags non-finite input coordinates (kStatusNonFinite)
int launch_normalize(double* out, const double* in, int n, const CellGeom& g, cudaStream_t st,
                     int* status = nullptr);
int launch_extend(double* cext, int* text, int* mapping, const double* coord, const int* atype,
                  int nloc, int nshift, const double* svec_dev, cudaStream_t st);
size_t nlist_pt_workspace(int nloc, const CellGeom& g);
int launch_nlist_pt(int* nlist, const double* coord, const int* atype, int nloc, const CellGeom& g,
                    const int* shift_pos_dev, const double* svec_dev, double rcut,
                    const SelInfo& sel, void* workspace, int* status, cudaStream_t st,
                    const int* gate = nullptr);
int launch_format_nlist(int* nlist, const double* coord, const int* atype, const int* rows, int nall,
                        const int* counts, int max_nbor, int nloc, double rcut, const SelInfo& sel,
                        int* status, cudaStream_t st);
// Many periodic frames of different sizes in one set of launches: frame f
// owns atoms [atom_off[f], atom_off[f+1]) of the concatenated arrays, cells
// [cell_off[f], cell_off[f+1]) of one global cell list, image shifts
// shift_pos[spos_off[f] ..] / svec[3 * svec_off[f] ..], geometry geom[f].
// Extended indices in the lists stay per frame: s * natoms_f + j_local.
struct FrameTab {
  int nframes;
  const int* atom_off;
  const int* cell_off;
  const int* spos_off;
  const int* svec_off;
  const CellGeom* geom;
};

__device__ __forceinline__ int frame_of(const int* off, int nframes, int x) {
  int lo = 0, hi = nframes;  // off[lo] <= x < off[hi]
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (off[mid] <= x) lo = mid; else hi = mid;
  }
  return lo;
}

size_t nlist_batch_workspace(int natoms, int ncells);
// wrap (normalize) and build the typed lists of every frame: coord_out
// receives the wrapped coordinates; nlist [natoms, sum(sel)]
int launch_nlist_batch(int* nlist, double* coord_out, const double* coord_in, const int* atype, int natoms,
                       int ncells, const FrameTab& ft, const double* svec, const int* shift_pos, double rcut,
                       const SelInfo& sel, void* workspace, int* status, cudaStream_t st);

// external list with explicit ghosts (CSR over the local atoms) -> typed list
int launch_format_ext(int* nlist, const double* coord_ext, const int* atype_ext, const int* off, const int* idx,
                      int nloc, int nall, double rcut, const SelInfo& sel, int sorted, int* status,
                      cudaStream_t st);
size_t transpose_workspace(long long npair, int nkeys);
int launch_transpose(Transpose& tr, const int* keys, long long npair, int nkeys, int mod,
                     void* workspace, int* status, cudaStream_t st);
int read_status(int* status_dev, cudaStream_t st, int out[kStatusSlots]);

// Skin lists: a candidate list of every pair within rcut + skin, built on
// wrapped coordinates, is reused over later evaluations; each evaluation
// selects the list at rcut from it.  gate[0] = rebuild in this evaluation,
// gate[1] = evaluations since the last build (-1: none).  The building
// kernels (cell list, candidate search) skip their work when gate[0] == 0.
// check: gate[0] = 1 when gate[1] is -1 or >= every, or an atom moved more
// than skin / 2 from its position at the build (ref)
int launch_skin_check(int* gate, const double* coord, const double* ref, int n, double skin, int every,
                      cudaStream_t st);
// build: out = wrapped coordinates, off = out - in, ref = in; reuse: out =
// in + off; outf / outflo = the FP32 high and low parts of out (the
// selection's prefilter and its split-FP32 displacements)
int launch_skin_coords(double* out, float4* outf, float4* outflo, double* off, double* ref, const double* in, int n,
                       const CellGeom& g, const int* gate, cudaStream_t st, int* status = nullptr);
// the list at rcut from the candidate rows [nloc, ncand] (extended indices
// s * nloc + j, -1 padding): the same ranking and per-type placement as a
// fresh build on the same coordinates.  margin: FP32 prefilter radius above
// rcut (covers the FP32 rounding of coordinates and shifts)
int launch_skin_select(int* nlist, const int* cand, int ncand, const double* coord, const float4* coordf,
                       const float4* coordflo, const int* atype, const double* svec, const float4* svecf,
                       const float4* svecflo, int nloc, double rcut, double margin, const SelInfo& sel, int* status,
                       cudaStream_t st);
// gate[1] = gate[0] ? 1 : gate[1] + 1; gate[0] = 0
int launch_skin_advance(int* gate, cudaStream_t st);
int sel_from_host(const int* sel_host, int ntypes, SelInfo& s);

}  // namespace dpgb
