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

// navigation kernels (kernels_nav.cu); mixed = FP32-interval box decisions
cudaError_t launch_step(const GeomView &g, const StepArgs &a, bool mixed, cudaStream_t s);
cudaError_t launch_safety(const GeomView &g, int64_t n, const double *px, const double *py, const double *pz,
                          const vgn_state *in, double *safety, bool mixed, int max_blocks, cudaStream_t s);
cudaError_t launch_locate(const GeomView &g, int64_t n, const double *px, const double *py, const double *pz,
                          vgn_state *out, bool mixed, int max_blocks, cudaStream_t s);
cudaError_t launch_shape_fp64(int op, int type, const double *row, int64_t n, const double *px, const double *py,
                              const double *pz, const double *dx, const double *dy, const double *dz, double *out,
                              int max_blocks, cudaStream_t s);

}  // namespace vgn
