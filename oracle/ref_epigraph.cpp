// Host build of the reference's epigraph projection kernel `epigraphproj`
// with its active-set QP `solve_qp` (opymize/operators/proj.cu:222-831), used
// ONLY as a test oracle.  The reference source is included where it lies; the
// CUDA qualifiers are defined away, the compile-time constants the reference
// bakes in (proj.py:436-460) become globals set per call, and the kernel runs
// once per instance (j, i) with a one-thread "block" at (i, j).
#include <math.h>
#include <stdint.h>
#include <stdio.h>

typedef unsigned int uint;

#define __device__
#define __global__ static
#define EPIGRAPH_PROJ 1
#define TYPE_T double
#define FABS fabs

#ifndef ndim
#error "compile with -Dndim=1|2|3"
#endif

static int ref_maxiter, ref_nfuns, ref_nregions, ref_npoints, ref_nsub;
static const unsigned char* ref_I;
static const int64_t* ref_J;
static double* ref_A;
static double* ref_B;

#define term_maxiter ref_maxiter
#define term_tolerance 1e-9
#define nfuns ref_nfuns
#define nregions ref_nregions
#define npoints ref_npoints
#define nsubpoints ref_nsub
#define I ref_I
#define J ref_J
#define A_STORE ref_A
#define B_STORE ref_B

struct ref_dim3 { int x, y, z; };
static ref_dim3 blockIdx, blockDim, threadIdx;

#include "proj.cu"

#undef I
#undef J

// x: (nregions, nfuns_, ndim+1) in place; Ib: (nfuns_, npoints_) bytes;
// Jb: (nregions_, nsub_) int64; v: (npoints_, ndim); b: (nfuns_, npoints_).
extern "C" void ref_epigraph_proj(double* x, const unsigned char* Ib, const int64_t* Jb,
                                  double* v, double* b, int nfuns_, int nregions_,
                                  int npoints_, int nsub_) {
  ref_I = Ib;
  ref_J = Jb;
  ref_A = v;
  ref_B = b;
  ref_nfuns = nfuns_;
  ref_nregions = nregions_;
  ref_npoints = npoints_;
  ref_nsub = nsub_;
  ref_maxiter = ndim * nsub_;
  blockDim.x = blockDim.y = blockDim.z = 1;
  threadIdx.x = threadIdx.y = threadIdx.z = 0;
  for (int j = 0; j < nregions_; ++j)
    for (int i = 0; i < nfuns_; ++i) {
      blockIdx.x = i;
      blockIdx.y = j;
      epigraphproj(x);
    }
}

extern "C" int ref_epigraph_ndim(void) { return ndim; }
