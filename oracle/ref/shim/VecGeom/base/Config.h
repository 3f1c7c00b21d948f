// VecGeom/base/Config.h -- hand-written configuration header for the CPU
// reference build under oracle/_ref (test infrastructure).  The reference
// generates this file from VecGeom/base/Config.h.in with cmake; these are the
// options of its default CUDA-capable build, minus CUDA, Vc, ROOT, Geant4, GDML:
//   scalar backend, double precision, no volume specialisation
//   (CMakeLists.txt:155), in-place transformations, the PlaneShell
//   trapezoid (CMakeLists.txt:156) and the index navigation state
//   (VECGEOM_USE_NAVINDEX, forced ON by CUDA builds, CMakeLists.txt:163-166) with
//   index-valued path states (VECGEOM_USE_INDEXEDNAVSTATES, ON by default,
//   CMakeLists.txt:161).
#ifndef VECGEOM_BASE_CONFIG_H_
#define VECGEOM_BASE_CONFIG_H_

#define VECGEOM_SCALAR
#define VECGEOM_CUDA_NO_VOLUME_SPECIALIZATION
#define VECGEOM_NO_SPECIALIZATION
#define VECGEOM_INPLACE_TRANSFORMATIONS
#define VECGEOM_PLANESHELL
#define VECGEOM_USE_NAVINDEX
#define VECGEOM_USE_INDEXEDNAVSTATES

#endif
