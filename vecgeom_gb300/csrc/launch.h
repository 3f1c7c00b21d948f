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
};

// all-FP64 kernels (kernels_fp64.cu)
cudaError_t launch_step_fp64(const GeomView &g, const StepArgs &a, cudaStream_t s);
cudaError_t launch_safety_fp64(const GeomView &g, int64_t n, const double *px, const double *py, const double *pz,
                               const vgn_state *in, double *safety, int max_blocks, cudaStream_t s);
cudaError_t launch_locate_fp64(const GeomView &g, int64_t n, const double *px, const double *py, const double *pz,
                               vgn_state *out, int max_blocks, cudaStream_t s);
cudaError_t launch_shape_fp64(int op, int type, const double *row, int64_t n, const double *px, const double *py,
                              const double *pz, const double *dx, const double *dy, const double *dz, double *out,
                              int max_blocks, cudaStream_t s);

}  // namespace vgn
