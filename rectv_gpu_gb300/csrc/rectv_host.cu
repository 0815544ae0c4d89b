// Host driver and C ABI of librectv_gb300.
//
// Replaces class rectv of the reference (src/include/rectv.cuh:7-55,
// src/cuda/rectv.cu:1-290) for one GPU.  Differences in mechanism, not in
// results:
//  * every buffer is device memory (no managed-memory streaming: the whole
//    state of the largest configuration fits in HBM), allocated at creation;
//  * chunks of nzp slices keep their own dual variables and z-halo semantics,
//    but several chunks are processed per kernel launch ("batch" of zb slices);
//  * an outer ADMM iteration is a fixed sequence of kernels and cuFFT calls
//    on one stream, captured once as a CUDA graph per buffer rotation and
//    replayed; rho lives on the device and is updated by a kernel, so the
//    host only reads the per-iteration log values (with one iteration of lag).
#include <cuda_runtime.h>
#include <cufft.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "rectv_gb300.h"
#include "handle.cuh"
#include "rectv_internal.cuh"
#include "tcgen05.cuh"

namespace rectv {

void cuda_check(cudaError_t e, const char *what, const char *file, int line) {
    if (e == cudaSuccess) return;
    const int code = (e == cudaErrorMemoryAllocation) ? RECTV_ERR_NOMEM : RECTV_ERR_CUDA;
    throw Error(code, std::string(what) + ": " + cudaGetErrorString(e) + " (" + file + ":" +
                          std::to_string(line) + ")");
}

void cufft_check(cufftResult e, const char *what, const char *file, int line) {
    if (e == CUFFT_SUCCESS) return;
    const int code = (e == CUFFT_ALLOC_FAILED) ? RECTV_ERR_NOMEM : RECTV_ERR_CUFFT;
    throw Error(code, std::string(what) + ": cufft error " + std::to_string((int)e) + " (" + file + ":" +
                          std::to_string(line) + ")");
}

std::string &last_error() {
    thread_local std::string msg;
    return msg;
}


__global__ void k_axpy(float *y, const float *x, float a, long long count) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < count) y[i] += a * x[i];
}

void Handle::launch_axpy(float *y, const float *x, float a, long long count) {
    k_axpy<<<(unsigned)((count + 255) / 256), 256, 0, stream>>>(y, x, a, count);
    LAUNCH_CHECK("k_axpy");
}

}  // namespace rectv

// ===========================================================================
// C ABI
// ===========================================================================
struct rectv_handle {
    rectv::Handle *h;
    int n, ntheta, m, nz, nzp, ngpus;
};

namespace {

rectv::Handle *live(rectv_handle *h) {
    if (!h) throw rectv::Error(RECTV_ERR_ARG, "rectv: null handle");
    if (!h->h || h->h->freed) throw rectv::Error(RECTV_ERR_STATE, "rectv: object was freed");
    return h->h;
}

}  // namespace

extern "C" {

const char *rectv_last_error(void) { return rectv::last_error().c_str(); }

const char *rectv_version(void) { return "rectv_gb300 1.0 (sm_103a)"; }

int rectv_create(int n, int ntheta, int m, int nz, int nzp, int ngpus, rectv_handle **out) {
    return rectv::guarded([&] {
        if (!out) throw rectv::Error(RECTV_ERR_ARG, "rectv_create: null output");
        *out = nullptr;
        auto *hh = new rectv::Handle(n, ntheta, m, nz, nzp, ngpus);
        auto *w = new rectv_handle{hh, n, ntheta, m, nz, nzp, hh->ngpus};
        *out = w;
    });
}

int rectv_get_dims(const rectv_handle *h, int *n, int *ntheta, int *m, int *nz, int *nzp, int *ngpus) {
    return rectv::guarded([&] {
        if (!h) throw rectv::Error(RECTV_ERR_ARG, "rectv: null handle");
        if (n) *n = h->n;
        if (ntheta) *ntheta = h->ntheta;
        if (m) *m = h->m;
        if (nz) *nz = h->nz;
        if (nzp) *nzp = h->nzp;
        if (ngpus) *ngpus = h->ngpus;
    });
}

int rectv_run(rectv_handle *h, float *fres, const float *g, const float *theta, const float *phi, float center,
              float lambda0, float lambda1, int niter, int titer) {
    return rectv::guarded([&] {
        rectv::Handle *H = live(h);
        if (!fres || !g || !theta || !phi) throw rectv::Error(RECTV_ERR_ARG, "rectv_run: null pointer");
        CUDA_CHECK(cudaMemcpyAsync(H->gdata, g, sizeof(float) * (size_t)H->nz * H->ntheta * H->n,
                                   cudaMemcpyHostToDevice, H->stream));
        H->setup(theta, phi, center, lambda0, lambda1, titer);
        H->iterate(niter);
        const size_t nf = (size_t)H->nzc * H->slab;
        CUDA_CHECK(cudaMemcpyAsync(fres, H->U[H->cur], sizeof(float) * nf, cudaMemcpyDeviceToHost, H->stream));
        CUDA_CHECK(cudaStreamSynchronize(H->stream));
        const size_t total = (size_t)H->nz * H->slab;
        if (total > nf) std::memset(fres + nf, 0, sizeof(float) * (total - nf));
    });
}

int rectv_check_adjoints(rectv_handle *h, double *res, const float *g, const float *theta, const float *phi,
                         float lambda1, float center) {
    return rectv::guarded([&] {
        rectv::Handle *H = live(h);
        if (!res || !g || !theta || !phi) throw rectv::Error(RECTV_ERR_ARG, "rectv_check_adjoints: null pointer");
        H->check_adjoints(res, g, theta, phi, lambda1, center);
    });
}

int rectv_free(rectv_handle *h) {
    return rectv::guarded([&] {
        if (!h) throw rectv::Error(RECTV_ERR_ARG, "rectv: null handle");
        if (h->h) {
            delete h->h;
            h->h = nullptr;
        }
    });
}

void rectv_destroy(rectv_handle *h) {
    if (!h) return;
    if (h->h) delete h->h;
    delete h;
}

int rectv_set_verbose(rectv_handle *h, int verbose) {
    return rectv::guarded([&] { live(h)->verbose = verbose != 0; });
}

int rectv_set_graphs(rectv_handle *h, int enable) {
    return rectv::guarded([&] {
        rectv::Handle *H = live(h);
        H->use_graphs = enable != 0;
        H->drop_graphs();
    });
}

int rectv_setup_device(rectv_handle *h, const float *d_g, const float *d_theta, const float *d_phi, float center,
                       float lambda0, float lambda1, int titer) {
    return rectv::guarded([&] {
        rectv::Handle *H = live(h);
        std::vector<float> th(H->ntheta), ph((size_t)2 * H->ntheta * H->m);
        CUDA_CHECK(cudaMemcpyAsync(H->gdata, d_g, sizeof(float) * (size_t)H->nz * H->ntheta * H->n,
                                   cudaMemcpyDeviceToDevice, H->stream));
        CUDA_CHECK(cudaMemcpyAsync(th.data(), d_theta, sizeof(float) * th.size(), cudaMemcpyDeviceToHost, H->stream));
        CUDA_CHECK(cudaMemcpyAsync(ph.data(), d_phi, sizeof(float) * ph.size(), cudaMemcpyDeviceToHost, H->stream));
        CUDA_CHECK(cudaStreamSynchronize(H->stream));
        H->setup(th.data(), ph.data(), center, lambda0, lambda1, titer);
    });
}

int rectv_iterate(rectv_handle *h, int niter) {
    return rectv::guarded([&] { live(h)->iterate(niter); });
}

int rectv_get_result_device(rectv_handle *h, float *d_f) {
    return rectv::guarded([&] {
        rectv::Handle *H = live(h);
        const size_t nf = (size_t)H->nzc * H->slab;
        CUDA_CHECK(cudaMemcpyAsync(d_f, H->U[H->cur], sizeof(float) * nf, cudaMemcpyDeviceToDevice, H->stream));
        const size_t total = (size_t)H->nz * H->slab;
        if (total > nf) CUDA_CHECK(cudaMemsetAsync(d_f + nf, 0, sizeof(float) * (total - nf), H->stream));
    });
}

int rectv_get_stream(rectv_handle *h, void **stream) {
    return rectv::guarded([&] {
        if (!stream) throw rectv::Error(RECTV_ERR_ARG, "rectv_get_stream: null output");
        *stream = (void *)live(h)->stream;
    });
}

int rectv_synchronize(rectv_handle *h) {
    return rectv::guarded([&] { live(h)->check_device_errors(); });
}

int rectv_get_history(rectv_handle *h, double *rdiff, double *rho, double *r, double *s, int *count) {
    return rectv::guarded([&] {
        rectv::Handle *H = live(h);
        if (!count) throw rectv::Error(RECTV_ERR_ARG, "rectv_get_history: null count");
        const int cap = *count;
        const int nrec = (int)H->h_rdiff.size();
        for (int i = 0; i < std::min(cap, nrec); ++i) {
            if (rdiff) rdiff[i] = H->h_rdiff[i];
            if (rho) rho[i] = H->h_rho[i];
            if (r) r[i] = H->h_r[i];
            if (s) s[i] = H->h_s[i];
        }
        *count = nrec;
    });
}

int rectv_op_set_geometry(rectv_handle *h, const float *d_theta, const float *d_phi, float center) {
    return rectv::guarded([&] {
        rectv::Handle *H = live(h);
        std::vector<float> th(H->ntheta), ph((size_t)2 * H->ntheta * H->m);
        CUDA_CHECK(cudaMemcpyAsync(th.data(), d_theta, sizeof(float) * th.size(), cudaMemcpyDeviceToHost, H->stream));
        CUDA_CHECK(cudaMemcpyAsync(ph.data(), d_phi, sizeof(float) * ph.size(), cudaMemcpyDeviceToHost, H->stream));
        CUDA_CHECK(cudaStreamSynchronize(H->stream));
        H->session = false;
        H->set_geometry(th.data(), ph.data(), center);
    });
}

int rectv_op_radonapr(rectv_handle *h, float *d_g, const float *d_f, int nslices, float tau) {
    return rectv::guarded([&] {
        rectv::Handle *H = live(h);
        if (!H->gd.sincos) throw rectv::Error(RECTV_ERR_STATE, "rectv_op_radonapr: set geometry first");
        if (nslices < 1 || nslices > H->nz) throw rectv::Error(RECTV_ERR_ARG, "rectv_op_radonapr: bad nslices");
        H->session = false;
        H->op_forward(d_g, d_f, nslices, tau);
        CUDA_CHECK(cudaStreamSynchronize(H->stream));
    });
}

int rectv_op_radonapradj(rectv_handle *h, float *d_f, const float *d_g, int nslices, float tau) {
    return rectv::guarded([&] {
        rectv::Handle *H = live(h);
        if (!H->gd.sincos) throw rectv::Error(RECTV_ERR_STATE, "rectv_op_radonapradj: set geometry first");
        if (nslices < 1 || nslices > H->nz) throw rectv::Error(RECTV_ERR_ARG, "rectv_op_radonapradj: bad nslices");
        H->session = false;
        H->op_adjoint(d_f, d_g, nslices, tau);
        CUDA_CHECK(cudaStreamSynchronize(H->stream));
    });
}

int rectv_op_gradient(rectv_handle *h, float *d_h2, const float *d_fm, float lambda1, int flgl, int flgr) {
    return rectv::guarded([&] {
        rectv::Handle *H = live(h);
        rectv::TvGeo t = H->tv;
        t.nchunks = 1;
        t.lambda1 = lambda1;
        t.sg = (float)(1.0 / (2.0 * std::cbrt(2.0) * ((double)lambda1 / 2.0)));
        t.sd = (float)(1.0 / (4.0 * std::cbrt(2.0) * ((double)lambda1 / 2.0)));
        rectv::launch_gradient_ref(d_fm, 1, d_h2, flgl ? 1 : 0, flgr ? 1 : 0, t, H->stream);
        CUDA_CHECK(cudaStreamSynchronize(H->stream));
    });
}

int rectv_op_divergent(rectv_handle *h, float *d_fn, const float *d_h2, float lambda1, float tau) {
    return rectv::guarded([&] {
        rectv::Handle *H = live(h);
        rectv::TvGeo t = H->tv;
        t.nchunks = 1;
        t.lambda1 = lambda1;
        t.sg = (float)(1.0 / (2.0 * std::cbrt(2.0) * ((double)lambda1 / 2.0)));
        t.sd = (float)(1.0 / (4.0 * std::cbrt(2.0) * ((double)lambda1 / 2.0)));
        rectv::launch_divergent_ref(d_fn, d_h2, tau, t, H->stream);
        CUDA_CHECK(cudaStreamSynchronize(H->stream));
    });
}

}  // extern "C"

extern "C" {

int rectv_fbp(rectv_handle *h, float *frec, const float *g, const float *theta, float center) {
    return rectv::guarded([&] {
        rectv::Handle *H = live(h);
        if (!frec || !g || !theta) throw rectv::Error(RECTV_ERR_ARG, "rectv_fbp: null pointer");
        H->fbp(frec, g, theta, center);
    });
}

int rectv_run_init(rectv_handle *h, float *fres, const float *g, const float *theta, const float *phi,
                   const float *finit, float center, float lambda0, float lambda1, int niter, int titer) {
    return rectv::guarded([&] {
        rectv::Handle *H = live(h);
        if (!fres || !g || !theta || !phi) throw rectv::Error(RECTV_ERR_ARG, "rectv_run_init: null pointer");
        CUDA_CHECK(cudaMemcpyAsync(H->gdata, g, sizeof(float) * (size_t)H->nz * H->ntheta * H->n,
                                   cudaMemcpyHostToDevice, H->stream));
        H->setup(theta, phi, center, lambda0, lambda1, titer, finit);
        H->iterate(niter);
        const size_t nf = (size_t)H->nzc * H->slab;
        CUDA_CHECK(cudaMemcpyAsync(fres, H->U[H->cur], sizeof(float) * nf, cudaMemcpyDeviceToHost, H->stream));
        CUDA_CHECK(cudaStreamSynchronize(H->stream));
        const size_t total = (size_t)H->nz * H->slab;
        if (total > nf) std::memset(fres + nf, 0, sizeof(float) * (total - nf));
    });
}

int rectv_preprocess(float *out, const void *data, const void *dark, const void *flat, int dtype, int ntheta, int nz,
                     int n, int ndark, int nflat) {
    return rectv::guarded([&] { rectv::preprocess(out, data, dark, flat, dtype, ntheta, nz, n, ndark, nflat); });
}

int rectv_launch_kernel(rectv_handle *h, int which, int reps) {
    return rectv::guarded([&] { live(h)->launch_kernel(which, reps); });
}

int rectv_kernel_cost(rectv_handle *h, int which, double *bytes, double *flops) {
    return rectv::guarded([&] {
        if (!bytes || !flops) throw rectv::Error(RECTV_ERR_ARG, "rectv_kernel_cost: null output");
        live(h)->kernel_cost(which, bytes, flops);
    });
}

}  // extern "C"

namespace rectv {
// FP32 FMA throughput: 8 independent chains per thread of scalar fma.rn
// (packed = 0) or packed fma.rn.f32x2 (packed = 1), enough blocks to fill
// every SM; the result is written so that the chains are not removed.
__global__ void k_fma_peak(float *out, int iters, int packed) {
    float2 a[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) a[i] = make_float2(threadIdx.x * 1e-7f + i, blockIdx.x * 1e-7f - i);
    const float2 b = make_float2(0.999999f, 0.999998f), c = make_float2(1e-7f, 2e-7f);
    if (packed) {
        for (int k = 0; k < iters; ++k)
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                unsigned long long d;
                asm volatile("fma.rn.f32x2 %0, %1, %2, %3;"
                             : "=l"(d)
                             : "l"(*reinterpret_cast<const unsigned long long *>(&a[i])),
                               "l"(*reinterpret_cast<const unsigned long long *>(&b)),
                               "l"(*reinterpret_cast<const unsigned long long *>(&c)));
                a[i] = *reinterpret_cast<const float2 *>(&d);
            }
    } else {
        for (int k = 0; k < iters; ++k)
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                a[i].x = fmaf(a[i].x, b.x, c.x);
                a[i].y = fmaf(a[i].y, b.y, c.y);
            }
    }
    float s = 0.f;
#pragma unroll
    for (int i = 0; i < 8; ++i) s += a[i].x + a[i].y;
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
}  // namespace rectv

extern "C" int rectv_measure_fp32_peak(double *tflops_fma, double *tflops_fma2) {
    return rectv::guarded([&] {
        if (!tflops_fma || !tflops_fma2) throw rectv::Error(RECTV_ERR_ARG, "rectv_measure_fp32_peak: null output");
        int dev = 0, nsm = 0;
        CUDA_CHECK(cudaGetDevice(&dev));
        CUDA_CHECK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
        const int threads = 256, blocks = nsm * 8, iters = 4096;
        float *out = nullptr;
        cudaStream_t s = nullptr;
        cudaEvent_t a = nullptr, b = nullptr;
        CUDA_CHECK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
        CUDA_CHECK(cudaMallocAsync(&out, sizeof(float) * threads * blocks, s));
        CUDA_CHECK(cudaEventCreate(&a));
        CUDA_CHECK(cudaEventCreate(&b));
        for (int packed = 0; packed < 2; ++packed) {
            float best = 1e30f;
            for (int rep = 0; rep < 4; ++rep) {  // the first launch warms up; best of the rest
                CUDA_CHECK(cudaEventRecord(a, s));
                rectv::k_fma_peak<<<blocks, threads, 0, s>>>(out, iters, packed);
                LAUNCH_CHECK("k_fma_peak");
                CUDA_CHECK(cudaEventRecord(b, s));
                CUDA_CHECK(cudaEventSynchronize(b));
                float ms = 0.f;
                CUDA_CHECK(cudaEventElapsedTime(&ms, a, b));
                if (rep > 0) best = std::min(best, ms);
            }
            const double flops = 2.0 * 16 * (double)iters * threads * blocks;  // 16 FMAs per thread and iteration
            (packed ? *tflops_fma2 : *tflops_fma) = flops / (best * 1e-3) / 1e12;
        }
        CUDA_CHECK(cudaFreeAsync(out, s));
        CUDA_CHECK(cudaStreamSynchronize(s));
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        cudaStreamDestroy(s);
    });
}

namespace rectv {
// One block waits on an mbarrier that nothing arrives on: first for `limit`
// cycles, then nwait - 1 more times as the kernels' later waits do after an
// expiry (healthy = false), and records the expiry in the handle's device
// error counter, as the kernels do.  Nothing is in flight, so the context
// stays usable.
__global__ void k_wait_probe(int *err, long long limit, int nwait) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        tc::mbar_init(&bar, 1);
        tc::fence_mbar_init();
    }
    __syncthreads();
    bool ok = tc::mbar_wait(&bar, 0u, true, limit);
    for (int i = 1; i < nwait; ++i) ok = tc::mbar_wait(&bar, 0u, ok) && ok;
    if (!ok && threadIdx.x == 0) atomicAdd(err, 1);
}
}  // namespace rectv

extern "C" {

int rectv_autotune(rectv_handle *h, int force, int *zper, int *sc_grid) {
    return rectv::guarded([&] {
        rectv::Handle *H = live(h);
        if (!H->session) throw rectv::Error(RECTV_ERR_STATE, "rectv_autotune: needs a set-up session");
        const rectv::Tune t = rectv::autotune(*H, force != 0);
        if (zper) *zper = t.zper;
        if (sc_grid) *sc_grid = t.sc_grid;
    });
}

int rectv_get_device_bytes(rectv_handle *h, double *bytes) {
    return rectv::guarded([&] {
        if (!bytes) throw rectv::Error(RECTV_ERR_ARG, "rectv_get_device_bytes: null output");
        *bytes = (double)live(h)->device_bytes();
    });
}

int rectv_selftest_wait(rectv_handle *h, long long limit_cycles, int nwait) {
    return rectv::guarded([&] {
        rectv::Handle *H = live(h);
        if (limit_cycles < 1 || limit_cycles > rectv::tc::kWaitLong || nwait < 1 || nwait > 100000)
            throw rectv::Error(RECTV_ERR_ARG, "rectv_selftest_wait: 1 <= limit_cycles <= 2e9, 1 <= nwait <= 1e5");
        rectv::k_wait_probe<<<1, 32, 0, H->stream>>>(H->gd.err, limit_cycles, nwait);
        LAUNCH_CHECK("k_wait_probe");
    });
}

int rectv_get_launch_counts(rectv_handle *h, int *kernels, int *fft_execs, int *batch_slices) {
    return rectv::guarded([&] {
        rectv::Handle *H = live(h);
        int k = 0, f = 0;
        H->launch_counts(&k, &f);
        if (kernels) *kernels = k;
        if (fft_execs) *fft_execs = f;
        if (batch_slices) *batch_slices = H->zb;
    });
}

int rectv_get_directions(rectv_handle *h, int *ndir, int *nrays) {
    return rectv::guarded([&] {
        rectv::Handle *H = live(h);
        if (ndir) *ndir = H->gd.dirs ? H->gd.ndir : 0;
        if (nrays) *nrays = H->ntheta;
    });
}

int rectv_plan_directions(const float *theta, int n, int ntheta, double tol_cells, double min_group, int *ndir,
                          int *max_rays) {
    return rectv::guarded([&] {
        if (!theta) throw rectv::Error(RECTV_ERR_ARG, "rectv_plan_directions: null pointer");
        if (n < 2 || ntheta < 1) throw rectv::Error(RECTV_ERR_ARG, "rectv_plan_directions: bad sizes");
        rectv::DirPlan dp;
        const bool used = rectv::build_dir_plan(theta, n, ntheta, 16, rectv::dir_fwd_capacity(),
                                                tol_cells > 0 ? tol_cells : rectv::kDirTolCells,
                                                min_group > 0 ? min_group : rectv::kDirMinGroup, dp);
        int mr = 0;
        for (size_t d = 0; d + 1 < dp.ray_start.size(); ++d) mr = std::max(mr, dp.ray_start[d + 1] - dp.ray_start[d]);
        if (ndir) *ndir = used ? dp.ndir : 0;
        if (max_rays) *max_rays = mr;
    });
}

}  // extern "C"

// ===========================================================================
// Allocation-free ADMM shrink step.
//
// Some callers cannot let a library allocate device memory: an application
// that owns the whole device budget through its own pool and hands this code
// only its buffers, or a processing loop that must not stall, since
// cudaMalloc/cudaFree can synchronise the device and can fail at run time
// when memory is fragmented.  rectv_shrink_noalloc serves them: the caller
// passes every input and output, and the only scratch (the FP64 per-block
// partial sums of the residual norms, and the rho value the kernel reads from
// device memory) lives in the file-scope array below, which every GPU that
// loads this library holds until the process exits.
// ===========================================================================
namespace rectv {
namespace {

// At most this many thread blocks per call: 3 doubles of partial sums each.
constexpr int kNoAllocMaxBlocks = 65536;
constexpr int kNoAllocRhoSlot = 3 * kNoAllocMaxBlocks;  // one double slot holds rho
static __device__ __align__(256) double g_noalloc_scratch[3 * kNoAllocMaxBlocks + 2];

constexpr int kNoAllocMaxDevices = 256;
std::mutex g_noalloc_mu;
double *g_noalloc_ptr[kNoAllocMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device.  The first call
// on a device looks it up (host code cannot use the symbol itself as a device
// address); that first call should therefore come before any stream capture.
// The address is kept for the life of the process: it belongs to the
// device's primary context, so after a cudaDeviceReset of that device it is
// stale and this entry point must not be used on that device again.
double *noalloc_scratch(cudaStream_t s) {
    int dev = 0;
    CUDA_CHECK(cudaGetDevice(&dev));
    if (s) {
        int sdev = -1;
        CUDA_CHECK(cudaStreamGetDevice(s, &sdev));
        if (sdev != dev)
            throw Error(RECTV_ERR_ARG, "rectv_shrink_noalloc: the stream belongs to device " + std::to_string(sdev) +
                                           ", the current device is " + std::to_string(dev) +
                                           "; make the stream's device current");
    }
    if (dev < 0 || dev >= kNoAllocMaxDevices) throw Error(RECTV_ERR_ARG, "rectv_shrink_noalloc: device ordinal out of range");
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            throw Error(RECTV_ERR_CUDA, std::string("rectv_shrink_noalloc: cudaGetSymbolAddress failed: ") +
                                            cudaGetErrorString(e));
        g_noalloc_ptr[dev] = static_cast<double *>(p);
    }
    return g_noalloc_ptr[dev];
}

__global__ void k_noalloc_set_rho(float *dst, float rho) { *dst = rho; }

// Fixed-order FP64 sum of the partials: one block, each thread sums a strided
// share, then a tree over the threads.  The order differs from rectv_iterate's
// two-stage reduction (k_sum_stage1 over contiguous shares, then
// k_reduce_rho), so the sums agree with its history to FP64 rounding, not
// bit for bit.
__global__ void k_noalloc_sum3(const double *__restrict__ partials, int nparts, double *out) {
    __shared__ double sh[3][256];
    double a = 0, b = 0, c = 0;
    for (int i = threadIdx.x; i < nparts; i += blockDim.x) {
        a += partials[3 * i];
        b += partials[3 * i + 1];
        c += partials[3 * i + 2];
    }
    sh[0][threadIdx.x] = a;
    sh[1][threadIdx.x] = b;
    sh[2][threadIdx.x] = c;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) {
            sh[0][threadIdx.x] += sh[0][threadIdx.x + o];
            sh[1][threadIdx.x] += sh[1][threadIdx.x + o];
            sh[2][threadIdx.x] += sh[2][threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[0] = sh[0][0];
        out[1] = sh[1][0];
        out[2] = sh[2][0];
    }
}

}  // namespace
}  // namespace rectv

extern "C" int rectv_shrink_noalloc(const float *d_u_cur, const float *d_u_old, float *d_psi, float *d_mu, int n,
                                    int m, int nzp, int nchunks, float rho, float lambda0, float lambda1,
                                    double *d_sums, void *stream) {
    return rectv::guarded([&] {
        if (!d_u_cur || !d_u_old || !d_psi || !d_mu || !d_sums)
            throw rectv::Error(RECTV_ERR_ARG, "rectv_shrink_noalloc: null pointer");
        if (n < 2 || m < 1 || nzp < 1 || nchunks < 1)
            throw rectv::Error(RECTV_ERR_ARG, "rectv_shrink_noalloc: n>=2, m>=1, nzp>=1, nchunks>=1 required");
        if (!(rho > 0.f)) throw rectv::Error(RECTV_ERR_ARG, "rectv_shrink_noalloc: rho must be positive");
        rectv::TvGeo t{};
        t.n = n;
        t.m = m;
        t.nzp = nzp;
        t.nchunks = nchunks;
        t.vol_slab = (long long)n * n * m;
        t.gp = (long long)(n + 1) * (n + 1) * (m + 1) * (nzp + 1);
        t.comp_stride = (long long)nchunks * t.gp;
        t.lambda1 = lambda1;
        t.sg = (float)(1.0 / (2.0 * std::cbrt(2.0) * ((double)lambda1 / 2.0)));
        t.sd = (float)(1.0 / (4.0 * std::cbrt(2.0) * ((double)lambda1 / 2.0)));
        const long long gz = (long long)nchunks * (nzp + 1);
        if (gz > 65535)
            throw rectv::Error(RECTV_ERR_ARG, "rectv_shrink_noalloc: nchunks*(nzp+1) = " + std::to_string(gz) +
                                                  " exceeds the grid limit of 65535");
        const long long nblocks = (long long)((n + 1 + 31) / 32) * (long long)((n + 1 + 7) / 8) * gz;
        if (nblocks > rectv::kNoAllocMaxBlocks)
            throw rectv::Error(RECTV_ERR_ARG,
                               "rectv_shrink_noalloc: problem needs " + std::to_string(nblocks) +
                                   " thread blocks; the static scratch holds at most " +
                                   std::to_string(rectv::kNoAllocMaxBlocks) +
                                   " (ceil((n+1)/32)*ceil((n+1)/8)*nchunks*(nzp+1))");
        cudaStream_t s = static_cast<cudaStream_t>(stream);
        double *scratch = rectv::noalloc_scratch(s);
        float *rho_d = reinterpret_cast<float *>(scratch + rectv::kNoAllocRhoSlot);
        rectv::k_noalloc_set_rho<<<1, 1, 0, s>>>(rho_d, rho);
        LAUNCH_CHECK("k_noalloc_set_rho");
        const int nparts = rectv::launch_shrink(d_u_cur, d_u_old, d_psi, d_mu, rho_d, lambda0, 0, nchunks, t,
                                                scratch, s);
        rectv::k_noalloc_sum3<<<1, 256, 0, s>>>(scratch, nparts, d_sums);
        LAUNCH_CHECK("k_noalloc_sum3");
    });
}
