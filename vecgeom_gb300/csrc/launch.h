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
};

// track binning (kernels_sort.cu)
struct BinParams {
  float lo[3];     // world bounding box corner
  float scale[3];  // cells per mm along each axis
  int kbits;       // 2^kbits cells per axis, 1..6
};
size_t bin_scratch_words(int64_t n, int kbits);  // keys + histogram (perm not included)
cudaError_t launch_bin_tracks(int64_t n, const double *px, const double *py, const double *pz, const double *dx,
                              const double *dy, const double *dz, const BinParams &b, uint32_t *scratch,
                              uint32_t *perm, int max_blocks, cudaStream_t s);

// fixed device scratch of the allocation-free binned step (kernels_sort.cu)
size_t static_scratch_words();
cudaError_t static_scratch(uint32_t **ptr);  // current device's buffer

// navigation kernels (kernels_nav.cu); mixed = FP32-interval box decisions
cudaError_t launch_step(const GeomView &g, const StepArgs &a, bool mixed, int variant, cudaStream_t s);
int step_variant_count();
cudaError_t launch_safety(const GeomView &g, int64_t n, const double *px, const double *py, const double *pz,
                          const vgn_state *in, double *safety, bool mixed, int max_blocks, cudaStream_t s);
cudaError_t launch_locate(const GeomView &g, int64_t n, const double *px, const double *py, const double *pz,
                          vgn_state *out, bool mixed, int max_blocks, cudaStream_t s);
cudaError_t launch_shape_fp64(int op, int type, const double *row, int64_t n, const double *px, const double *py,
                              const double *pz, const double *dx, const double *dy, const double *dz, double *out,
                              int max_blocks, cudaStream_t s);

}  // namespace vgn
