// launch.h -- host-side launchers of the device kernels (one per kernel set).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/vgnav.h"
#include "geom_types.h"

namespace vgn {

struct StepArgs {
  int64_t n;
  const double *px, *py, *pz, *dx, *dy, *dz, *slimit;
  const vgn_state *in;
  vgn_state *out;
  double *step, *safety;
  int reloc;
  int max_blocks;
  const uint32_t *perm;  // optional visit order (track binning), nullptr = identity
  const uint32_t *perm_safety = nullptr;  // the safety pass's own order, nullptr = `perm`
};

// track binning (kernels_sort.cu)
struct BinParams {
  float lo[3];     // world bounding box corner
  float scale[3];  // cells per mm along each axis
  int kbits;       // 2^kbits cells per axis, 1..6
  int octants = 1; // 1: key = direction octant, then cell (the step's order); 0: cell only
};
constexpr size_t kScanSumWords = 512;             // tile sums of the histogram scan (kbits <= 6)
size_t bin_scratch_words(int64_t n, int kbits);  // keys + histogram + tile sums (perm not included)
cudaError_t launch_bin_tracks(int64_t n, const double *px, const double *py, const double *pz, const double *dx,
                              const double *dy, const double *dz, const BinParams &b, uint32_t *scratch,
                              uint32_t *perm, int max_blocks, cudaStream_t s);

// fixed device scratch of the allocation-free binned step (kernels_sort.cu)
size_t static_scratch_words();
cudaError_t static_scratch(uint32_t **ptr);  // current device's buffer

// one job of a multi-job launch: geometry view, SOA3D arrays and visit order
struct JobRec {
  GeomView g;
  const double *px, *py, *pz, *dx, *dy, *dz, *slimit;
  const vgn_state *in;
  vgn_state *out;
  double *step, *safety;
  const uint32_t *perm;  // nullptr = identity
  const uint32_t *perm_safety;  // the safety pass's own order, nullptr = `perm`
  int64_t n;
};
// the whole multi-job launch description, passed by value as a kernel parameter
struct JobTable {
  JobRec job[VGN_BATCH_MAX_JOBS];
  uint32_t chunk_begin[VGN_BATCH_MAX_JOBS + 1];  // first 32-track chunk of each job; [n_jobs] = total
  int32_t n_jobs;
};
static_assert(sizeof(JobTable) < 32000, "kernel parameters are limited to 32764 bytes");
// Navigation kernels (kernels_nav.cu), compiled three times: `sections` handles phi and theta
// sections, `full_ranges` leaves that code out (geometries whose shapes all span the full
// angular ranges), `booleans` adds the boolean solids to `full_ranges` (a geometry may not
// hold both booleans and sections).  The sets give identical results on the geometries they
// all handle.
namespace sections {
#include "launch_set.inc"
}  // namespace sections
namespace booleans {
#include "launch_set.inc"
}  // namespace booleans
namespace full_ranges {
#include "launch_set.inc"
}  // namespace full_ranges

}  // namespace vgn
