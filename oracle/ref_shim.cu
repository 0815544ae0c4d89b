// extern "C" entry points over the reference's class rectv, in place of its
// SWIG module (src/cuda/rectv.i:9-28), so that ctypes can drive the
// reference's own CUDA implementation.  TEST INFRASTRUCTURE ONLY: built by
// oracle/ref_build.py into oracle/_ref/librectv_ref.so and used as the
// "plain FP32" reference build (parity pin and timing baseline).
//
// Each function forwards its arguments unchanged: pointers are host
// addresses passed as size_t, as Solver does (src/rectv_gpu/solver.py:7-8,
// 82-83).  No free entry point is exported: rectv::free() ends with
// cudaDeviceReset() (rectv.cu:87), so callers run the reference in a process
// of its own and let process exit release it.
#include <cstddef>

#include "rectv.cuh"

extern "C" {

void *rectvref_create(int n, int ntheta, int m, int nz, int nzp, int ngpus) {
    return new rectv(n, ntheta, m, nz, nzp, ngpus);
}

void rectvref_run(void *h, float *fres, const float *g, const float *theta, const float *phi, float center,
                  float lambda0, float lambda1, int niter, int titer) {
    static_cast<rectv *>(h)->run((size_t)fres, (size_t)g, (size_t)theta, (size_t)phi, center, lambda0, lambda1,
                                 niter, titer);
}

void rectvref_check_adjoints(void *h, double *res, const float *g, const float *theta, const float *phi,
                             float lambda1, float center) {
    static_cast<rectv *>(h)->check_adjoints((size_t)res, (size_t)g, (size_t)theta, (size_t)phi, lambda1, center);
}

}  // extern "C"
