// struct Handle: the device state, geometry, cuFFT plans, captured graphs
// and host logic of one reconstruction problem (one rectv object of the
// reference, src/include/rectv.cuh:7-55, src/cuda/rectv.cu), shared by the
// C ABI (rectv_host.cu) and the multi-problem engine (engine.cu).
#pragma once

#include <cuda_runtime.h>
#include <cufft.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "rectv_gb300.h"
#include "rectv_internal.cuh"

namespace rectv {

// Message of the last failing C-ABI call on this thread.
std::string &last_error();

// Runs f, mapping exceptions to the C ABI's status codes and message.
template <class F>
int guarded(F &&f) {
    try {
        f();
        last_error().clear();
        return RECTV_OK;
    } catch (const Error &e) {
        last_error() = e.what();
        return e.code;
    } catch (const std::bad_alloc &) {
        last_error() = "host out of memory";
        return RECTV_ERR_NOMEM;
    } catch (const std::exception &e) {
        last_error() = e.what();
        return RECTV_ERR_ARG;
    }
}

namespace detail {


template <class T>
T *dalloc(size_t count, std::vector<void *> &owned, cudaStream_t s) {
    void *p = nullptr;
    if (count == 0) count = 1;
    // stream-ordered: freeing (cudaFreeAsync) never synchronises the device,
    // so problems can come and go while others run (engine.cu)
    CUDA_CHECK(cudaMallocAsync(&p, count * sizeof(T), s));
    owned.push_back(p);
    return static_cast<T *>(p);
}

inline int usfft_radius(int n, float *mu_out) {
    // radonusfft.cu:10-11
    const float eps = 1e-3f;
    const float mu = (float)(-std::log((double)eps) / (2.0 * n * (double)n));
    const double r = std::ceil(2.0 * n / kPiUsfft *
                               std::sqrt(-(double)mu * std::log((double)eps) + ((double)mu * n) * ((double)mu * n) / 4.0));
    *mu_out = mu;
    return (int)r;
}

}  // namespace detail

// Sizes of one problem's device buffers and its slice batch: a function of
// the dimensions, the per-batch scratch budget and the environment overrides
// (RECTV_SCATTER=direct, RECTV_CUFFT=1, RECTV_BATCH_BYTES), used both to
// allocate a handle and to estimate its device memory before creating it.
struct Layout {
    int P = 0, nchunks = 0, nzc = 0, zb = 0, nbatch = 0;
    bool tc_scatter = false;  // time samples mixed on the tensor cores in the adjoint (k_scatter_tc)
    bool pad_fft = false;     // hand-written padded-grid 2D FFTs
    bool fused_rows = false;  // fused residual rows (k_resid_rows)
    bool iter_plans = false;  // the outer iteration runs cuFFT plans
    long long slab = 0, gp = 0, img_spec = 0;
    size_t spec_elems = 0;
    double bytes = 0;         // estimate of all device memory, geometry included
};

inline Layout make_layout(int n, int ntheta, int m, int nz, int nzp, double batch_bytes) {
    Layout L;
    L.P = 2 * n;
    const long long P = L.P;
    L.nchunks = nz / nzp;
    L.nzc = L.nchunks * nzp;
    L.slab = (long long)n * n * m;
    L.gp = (long long)(n + 1) * (n + 1) * (m + 1) * (nzp + 1);
    // adjoint: tensor-core time-sample mixing (k_scatter_tc) from 8 time
    // samples up; RECTV_SCATTER=direct forces the FP32 scatter
    L.tc_scatter = m >= 8 && ntheta < 65536;  // ray index packed in 16 bits
    if (const char *e = std::getenv("RECTV_SCATTER"))
        if (!std::strcmp(e, "direct")) L.tc_scatter = false;
    {
        const char *e = std::getenv("RECTV_CUFFT");
        L.pad_fft = pad_fft_supported(L.P) && !(e && std::atoi(e) != 0);
    }
    L.fused_rows = L.pad_fft && resid_rows_supported(n);
    L.iter_plans = !(L.pad_fft && L.fused_rows && L.tc_scatter);
    const long long qp = n + 2 * kHalo + (n & 1);
    const long long img_fwd = (P + 2 * kHalo) * qp;
    // the tensor-core scatter fills Hermitian half planes (row pitch P/2+2),
    // the FP32 scatter full periodic planes
    L.img_spec = L.tc_scatter ? std::max(img_fwd, P * (P / 2 + 2)) : std::max(img_fwd, P * P);
    // batch size: largest zb = nzp*d, d | nchunks, with per-batch scratch under budget
    double budget = batch_bytes;
    if (budget <= 0) {
        budget = 40.0 * (1ull << 30);
        if (const char *e = std::getenv("RECTV_BATCH_BYTES")) budget = std::atof(e);
    }
    const double per_slice = (double)m * L.img_spec * 8.0 + (double)ntheta * n * 12.0;
    int d = 1;
    for (int cand = L.nchunks; cand >= 1; --cand) {
        if (L.nchunks % cand) continue;
        if (cand == 1 || per_slice * nzp * cand <= budget) {
            d = cand;
            break;
        }
    }
    L.zb = nzp * d;
    L.nbatch = L.nchunks / d;
    L.spec_elems = std::max<size_t>((size_t)L.zb * m * (size_t)L.img_spec,
                                    (size_t)2 * (n + 1) * (n + 1) * (m + 1) * (nzp + 1));
    const double nt = (double)ntheta * n;
    double b = 3.0 * L.nzc * L.slab * 4 + (double)nz * nt * 4 + 3.0 * 4 * L.nchunks * L.gp * 4;
    b += (double)L.zb * nt * 4 + L.spec_elems * 8.0 + (double)L.zb * ntheta * std::max(n, n / 2 + 1) * 8.0;
    if (L.fused_rows) b += (double)L.zb * ntheta * (n / 2 + 1) * 8.0;
    b += 3.0 * 8 * (double)((n + 32) / 32) * ((n + 8) / 8) * d * (nzp + 1) * L.nbatch + (4 << 20);
    // geometry: angle plan, adjoint entries (about 2.25 tiles per sample) and records
    b += nt * (4 + 2.5 * 4 + (L.tc_scatter ? 2.5 * 144 + 12 : 0)) + 8.0 * ntheta * m + (1 << 20);
    if (L.pad_fft) b += 16.0 * P * 8;
    // cuFFT work area when the iteration runs cuFFT (about one batch of 2D planes, at most 8 GiB)
    if (L.iter_plans) b += std::min(8.0 * (1ull << 30), (double)L.zb * m * P * P * 8.0);
    L.bytes = b;
    return L;
}

struct Handle {
    // dimensions (rectv.cuh:43-47)
    int n, ntheta, m, nz, nzp, ngpus, nchunks, nzc;
    int device = 0;
    bool freed = false;
    bool verbose = true;
    bool use_graphs = true;
    cudaStream_t stream = nullptr;      // where work is queued (bind_stream)
    cudaStream_t own_stream = nullptr;  // created with the handle, owns its allocations
    std::vector<void *> owned;

    Layout lay;
    double batch_bytes = -1;  // per-batch scratch budget (<= 0: default / RECTV_BATCH_BYTES)
    size_t dev_bytes = 0;     // device memory owned (buffers), and ...
    size_t geo_bytes = 0;     // ... held by the geometry
    UsGeo ug{};
    TvGeo tv{};
    float mu_us = 0.f;
    int zb = 0;        // slices per batch (multiple of nzp, divides nzc)
    int nbatch = 0;
    long long slab = 0;  // n*n*m
    long long gp = 0;    // dual points per chunk

    // device buffers
    float *U[3] = {nullptr, nullptr, nullptr};
    float *gdata = nullptr;
    float *psi = nullptr, *mu = nullptr;
    float *wdual = nullptr;  // w = mu - rho psi of the current outer iteration (psi's layout)
    float *h1 = nullptr;
    float2 *spec = nullptr;
    float2 *rows = nullptr;
    double *partials = nullptr;
    double *stage1 = nullptr;
    int nparts_batch = 0;
    double *dot_part = nullptr;
    double *dot_out = nullptr;
    float *rho_d = nullptr;
    int *iter_ctr = nullptr;
    double *stats = nullptr;
    int stats_cap = 0;
    GeoDev gd;
    std::vector<void *> geo_owned;

    // cuFFT
    cufftHandle p_r2c2d = 0, p_c2c2d = 0, p_rows_c2c = 0, p_rows_r2c = 0, p_c2r2d = 0;
    CUtensorMap spec_tmap;  // TMA boxes of the forward spectra (tensor-core gather)
    // key of the geometry on the device (set_geometry)
    bool geo_valid = false, geo_has_phi = false, geo_tc_scatter = false;
    float geo_center = 0.f, geo_tc_spr = 0.f;
    double geo_dir_min = 0.0, geo_dir_tol = 0.0;
    std::vector<float> geo_theta, geo_phi;
    // key of the captured graphs besides the geometry (setup)
    int graph_titer = -1;
    float graph_lambda0 = 0.f, graph_lambda1 = 0.f;
    bool plans_made = false;
    int img_per_fft = 0;
    void *fft_work = nullptr;
    // hand-written padded-grid FFTs (P a power of two in [256, 2048]) instead
    // of cuFFT + deapodise/pad + crop passes; RECTV_CUFFT=1 selects cuFFT
    bool pad_fft = false;
    float2 *fft_tw = nullptr;  // twiddle tables (pad_fft_twiddles)
    // fused residual rows (inverse row FFT, residual, R2C in one kernel)
    bool fused_rows = false;
    float2 *fft_tw_n = nullptr;  // twiddles of the n-point row transforms
    float2 *rows_adj = nullptr;  // the adjoint's row spectra [zb][ntheta][n/2+1]
    CUtensorMap fft_fwd_map, fft_inv_map;  // TMA tiles of the column passes

    // session
    bool session = false;
    int cur = 0;
    float lambda0 = 0.f, lambda1 = 1.f;
    int titer = 0;
    int iters_done = 0;
    int pending = 0;  // iterations queued by enqueue_iterations, not yet collected
    std::vector<double> h_rdiff, h_rho, h_r, h_s;
    double *stats_host = nullptr;  // pinned, allocated by the first iterate()
    int stats_host_cap = 0;
    cudaGraphExec_t graphs[3] = {nullptr, nullptr, nullptr};

    Handle(int n_, int ntheta_, int m_, int nz_, int nzp_, int ngpus_, double batch_bytes_ = -1) {
        batch_bytes = batch_bytes_;
        n = n_;
        ntheta = ntheta_;
        m = m_;
        nz = nz_;
        nzp = nzp_;
        if (n < 2 || ntheta < 1 || m < 1 || nz < 1 || nzp < 1)
            throw Error(RECTV_ERR_ARG, "rectv: n>=2, ntheta>=1, m>=1, nz>=1, nzp>=1 required");
        if (nzp > nz) throw Error(RECTV_ERR_ARG, "rectv: nzp must not exceed nz");
        if ((long long)n * ntheta >= (1LL << 32)) throw Error(RECTV_ERR_ARG, "rectv: n*ntheta too large");
        nchunks = nz / nzp;
        nzc = nchunks * nzp;
        ngpus = std::max(1, std::min(ngpus_, nchunks));  // rectv.cu:9
        CUDA_CHECK(cudaGetDevice(&device));
        const int r = detail::usfft_radius(n, &mu_us);
        if (r != kR) throw Error(RECTV_ERR_ARG, "rectv: USFFT radius " + std::to_string(r) + " != 4");
        try {
            init();
        } catch (...) {
            release();
            throw;
        }
    }

    ~Handle() { release(); }

    void init() {
        CUDA_CHECK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        own_stream = stream;
        usfft_prepare();
        gather_tc_prepare();
        scatter_tc_prepare();
        dir_prepare();
        pad_fft_prepare();
        const int P = 2 * n;
        ug.n = n;
        ug.ntheta = ntheta;
        ug.m = m;
        ug.P = P;
        ug.hp = P / 2 + 1;
        ug.hpitch = P / 2 + 1;
        ug.qp = n + 2 * kHalo + (n & 1);
        ug.qoff = (long long)kHalo * ug.qp + kHalo;
        ug.img_fwd = (long long)(P + 2 * kHalo) * ug.qp;
        ug.img_adj = (long long)P * P;
        ug.tn = (float)(2 * n);
        ug.inv2n = (float)(1.0 / (2.0 * n));
        ug.wexp = (float)(kPiUsfft * kPiUsfft / (double)mu_us);
        ug.cw = (float)(kPiUsfft / (double)mu_us / (double)n);
        ug.T = 16;
        ug.NT = (P + ug.T - 1) / ug.T;
        ug.zper = 64;
        ug.sc_grid = 0;

        lay = make_layout(n, ntheta, m, nz, nzp, batch_bytes);
        slab = lay.slab;
        gp = lay.gp;
        zb = lay.zb;
        nbatch = lay.nbatch;
        const int d = zb / nzp;

        for (int i = 0; i < 3; ++i) U[i] = alloc<float>((size_t)nzc * slab);
        gdata = alloc<float>((size_t)nz * ntheta * n);
        psi = alloc<float>((size_t)4 * nchunks * gp);
        mu = alloc<float>((size_t)4 * nchunks * gp);
        wdual = alloc<float>((size_t)4 * nchunks * gp);
        CUDA_CHECK(cudaMemsetAsync(wdual, 0, sizeof(float) * (size_t)4 * nchunks * gp, stream));
        h1 = alloc<float>((size_t)zb * ntheta * n);
        // spectra (forward images and the adjoint's half or full planes); also
        // the float4 gradient scratch of check_adjoints
        spec = alloc<float2>(lay.spec_elems);
        make_spec_tensor_map(&spec_tmap, spec, zb * m, ug);
        rows = alloc<float2>((size_t)zb * ntheta * (size_t)std::max(n, n / 2 + 1));

        tv.n = n;
        tv.m = m;
        tv.nzp = nzp;
        tv.nchunks = d;
        tv.vol_slab = slab;
        tv.gp = gp;
        tv.comp_stride = (long long)nchunks * gp;
        set_lambda1(1.0f);
        nparts_batch = shrink_blocks(tv, d);
        partials = alloc<double>((size_t)3 * nparts_batch * nbatch);
        dot_part = alloc<double>((size_t)dot_parts());
        dot_out = alloc<double>(8);
        stage1 = alloc<double>((size_t)3 * reduce_stage1_parts());
        rho_d = alloc<float>(1);
        iter_ctr = alloc<int>(1);
        gd.err = alloc<int>(1);
        CUDA_CHECK(cudaMemsetAsync(gd.err, 0, sizeof(int), stream));
        {
            pad_fft = lay.pad_fft;
            if (pad_fft) {
                const std::vector<float2> w = pad_fft_twiddles(P);
                fft_tw = alloc<float2>(w.size());
                CUDA_CHECK(cudaMemcpyAsync(fft_tw, w.data(), sizeof(float2) * w.size(), cudaMemcpyHostToDevice,
                                           stream));
                CUDA_CHECK(cudaStreamSynchronize(stream));
                ug.hpitch = P / 2 + 2;  // 16-byte half-plane rows for the TMA tiles
                make_pad_fft_maps(&fft_fwd_map, &fft_inv_map, spec, zb * m, ug);
                fused_rows = lay.fused_rows;
                if (fused_rows) {
                    const std::vector<float2> wn = pad_fft_twiddles(n);
                    fft_tw_n = alloc<float2>(wn.size());
                    CUDA_CHECK(cudaMemcpyAsync(fft_tw_n, wn.data(), sizeof(float2) * wn.size(),
                                               cudaMemcpyHostToDevice, stream));
                    rows_adj = alloc<float2>((size_t)zb * ntheta * (size_t)(n / 2 + 1));
                    CUDA_CHECK(cudaStreamSynchronize(stream));
                }
            }
        }
        CUDA_CHECK(cudaStreamSynchronize(stream));
    }

    // cuFFT plans are made on first need (never during stream capture): the
    // outer iteration needs them only off the hand-written path
    // (lay.iter_plans), the operator API, check_adjoints and FBP always.
    void ensure_plans() {
        if (!plans_made) make_fft_plans();
    }

    template <class T>
    T *alloc(size_t count) {
        T *p = detail::dalloc<T>(count, owned, stream);
        dev_bytes += std::max<size_t>(count, 1) * sizeof(T);
        return p;
    }

    size_t device_bytes() const { return dev_bytes + geo_bytes; }

    void set_lambda1(float l1) {
        lambda1 = l1;
        tv.lambda1 = l1;
        // kernels_operators.cuh:40-43 and 69-72
        tv.sg = (float)(1.0 / (2.0 * std::cbrt(2.0) * ((double)l1 / 2.0)));
        tv.sd = (float)(1.0 / (4.0 * std::cbrt(2.0) * ((double)l1 / 2.0)));
    }

    void make_fft_plans() {
        const int P = 2 * n;
        const double img_bytes = (double)P * P * 8.0;
        const int nimg = zb * m;
        int per = nimg;
        const double cap = 8.0 * (1ull << 30);
        while (per > 1 && per * img_bytes > cap) {
            int nx = per - 1;
            while (nx > 1 && nimg % nx) --nx;
            per = nx;
        }
        img_per_fft = per;
        size_t ws = 0, w1 = 0;
        CUFFT_CHECK(cufftCreate(&p_r2c2d));
        CUFFT_CHECK(cufftCreate(&p_c2c2d));
        CUFFT_CHECK(cufftCreate(&p_c2r2d));
        CUFFT_CHECK(cufftCreate(&p_rows_c2c));
        CUFFT_CHECK(cufftCreate(&p_rows_r2c));
        plans_made = true;
        for (cufftHandle h : {p_r2c2d, p_c2c2d, p_rows_c2c, p_rows_r2c, p_c2r2d})
            CUFFT_CHECK(cufftSetAutoAllocation(h, 0));
        {  // 2D R2C in place inside the padded forward images: real rows of
           // 2 qp floats -> P/2+1 complex of a qp-complex row
            int nn[2] = {P, P};
            int inem[2] = {P, 2 * ug.qp};
            int onem[2] = {P, ug.qp};
            CUFFT_CHECK(cufftMakePlanMany(p_r2c2d, 2, nn, inem, 1, (int)(2 * ug.img_fwd), onem, 1, (int)ug.img_fwd,
                                          CUFFT_R2C, per, &w1));
            ws = std::max(ws, w1);
        }
        {  // 2D C2R in place: Hermitian half planes of P/2+1 complex -> real rows of P+2 floats
            int nn[2] = {P, P};
            int inem[2] = {P, P / 2 + 1};
            int onem[2] = {P, P + 2};
            CUFFT_CHECK(cufftMakePlanMany(p_c2r2d, 2, nn, inem, 1, P * (P / 2 + 1), onem, 1, P * (P + 2), CUFFT_C2R,
                                          per, &w1));
            ws = std::max(ws, w1);
        }
        {  // 2D C2C full plane
            int nn[2] = {P, P};
            CUFFT_CHECK(cufftMakePlanMany(p_c2c2d, 2, nn, nullptr, 1, P * P, nullptr, 1, P * P, CUFFT_C2C, per,
                                          &w1));
            ws = std::max(ws, w1);
        }
        const int nrows = zb * ntheta;
        {  // rows C2C (forward operator's inverse transform)
            int nn[1] = {n};
            CUFFT_CHECK(cufftMakePlanMany(p_rows_c2c, 1, nn, nullptr, 1, n, nullptr, 1, n, CUFFT_C2C, nrows, &w1));
            ws = std::max(ws, w1);
        }
        {  // rows R2C in place (adjoint): 2(n/2+1) floats -> n/2+1 complex
            int nn[1] = {n};
            int inem[1] = {2 * (n / 2 + 1)};
            int onem[1] = {n / 2 + 1};
            CUFFT_CHECK(cufftMakePlanMany(p_rows_r2c, 1, nn, inem, 1, 2 * (n / 2 + 1), onem, 1, n / 2 + 1,
                                          CUFFT_R2C, nrows, &w1));
            ws = std::max(ws, w1);
        }
        if (ws > 0) fft_work = alloc<char>(ws);
        for (cufftHandle h : {p_r2c2d, p_c2c2d, p_rows_c2c, p_rows_r2c, p_c2r2d}) {
            CUFFT_CHECK(cufftSetWorkArea(h, fft_work));
            CUFFT_CHECK(cufftSetStream(h, stream));
        }
    }

    void drop_graphs() {
        for (auto &g : graphs)
            if (g) {
                cudaGraphExecDestroy(g);
                g = nullptr;
            }
    }

    void free_geo() {
        geo_valid = false;
        for (void *p : geo_owned) cudaFreeAsync(p, stream);
        geo_owned.clear();
        geo_bytes = 0;
        int *err = gd.err;
        gd = GeoDev();
        gd.err = err;
    }

    // Queue this handle's work on s (a stream of the same device) from now on;
    // nullptr returns to the handle's own stream.  The caller orders s after
    // the handle's earlier work (the engine binds only idle handles).
    void bind_stream(cudaStream_t s) {
        stream = s ? s : own_stream;
        if (plans_made)
            for (cufftHandle h : {p_r2c2d, p_c2c2d, p_rows_c2c, p_rows_r2c, p_c2r2d})
                CUFFT_CHECK(cufftSetStream(h, stream));
    }

    void release() {
        if (stream) cudaStreamSynchronize(stream);
        if (own_stream && own_stream != stream) cudaStreamSynchronize(own_stream);
        stream = own_stream;
        drop_graphs();
        free_geo();
        if (plans_made) {
            cufftDestroy(p_r2c2d);
            cufftDestroy(p_c2c2d);
            cufftDestroy(p_c2r2d);
            cufftDestroy(p_rows_c2c);
            cufftDestroy(p_rows_r2c);
            plans_made = false;
        }
        for (void *p : owned) cudaFreeAsync(p, stream);
        owned.clear();
        if (stats_host) cudaFreeHost(stats_host);
        stats_host = nullptr;
        stats_host_cap = 0;
        if (own_stream) cudaStreamDestroy(own_stream);
        stream = own_stream = nullptr;
        freed = true;
        session = false;
    }

    // 16 time samples per gather pass (the tensor-core gather's K)
    bool mp16() const { return m >= 8; }

    void check_live() const {
        if (freed) throw Error(RECTV_ERR_STATE, "rectv: object was freed");
    }

    // ---- geometry: angle plan, basis mixing matrix, centre shifts ----
    // Returns true when the geometry was (re)built: plan, K', shifts and
    // records are a function of (theta, phi, center) and of the kernel choice,
    // so a call with the same values keeps them (and the captured graphs).
    bool set_geometry(const float *theta_h, const float *phi_h, float center) {
        // gather items hold at most one sample table; scatter items are whole
        // tiles (one block owns each tile, so tiles are stored, never added)
        // forward items with >= 2 samples per ray use the tensor-core gather
        // (time samples are mixed once per ray); RECTV_GATHER=direct|tc forces
        // one kernel (A/B comparisons).  Below 8 time samples the direct
        // kernel's shared-memory rows are short and it stays the only one.
        float tc_min_spr = (mp16() ? 2.0f : -1.0f);
        if (const char *e = std::getenv("RECTV_GATHER")) {
            if (!std::strcmp(e, "direct")) tc_min_spr = -1.0f;
            if (!std::strcmp(e, "tc") && mp16()) tc_min_spr = 0.0f;
        }
        // adjoint: tensor-core time-sample mixing (k_scatter_tc) as fixed by
        // the layout at creation
        const bool tc_scatter = lay.tc_scatter;
        // direction path (dir_kernels.cu): rays that revisit a direction over
        // several half-turns share its sample positions, so the USFFT
        // interpolates once per position.  Used when the rays average at least
        // 2.5 per direction (RECTV_DIRS=1: whenever it can run, RECTV_DIRS=0:
        // never) and the adjoint fills Hermitian half planes; rays are grouped
        // when their samples agree within RECTV_DIR_TOL grid cells (2e-3).
        double dir_min = kDirMinGroup, dir_tol = kDirTolCells;
        if (const char *e = std::getenv("RECTV_DIRS")) {
            if (!std::strcmp(e, "0")) dir_min = -1.0;
            if (!std::strcmp(e, "1")) dir_min = 1.0;
        }
        if (const char *e = std::getenv("RECTV_DIR_TOL")) dir_tol = std::max(0.0, std::atof(e));
        if (!tc_scatter) dir_min = -1.0;
        const size_t nphi = phi_h ? (size_t)2 * m * ntheta : 0;
        if (geo_valid && center == geo_center && tc_min_spr == geo_tc_spr && tc_scatter == geo_tc_scatter &&
            dir_min == geo_dir_min && dir_tol == geo_dir_tol &&
            (phi_h != nullptr) == geo_has_phi && !std::memcmp(theta_h, geo_theta.data(), sizeof(float) * ntheta) &&
            (!phi_h || !std::memcmp(phi_h, geo_phi.data(), sizeof(float) * nphi)))
            return false;
        drop_graphs();
        free_geo();
        DirPlan dplan;
        const bool dirs =
            dir_min > 0 && build_dir_plan(theta_h, n, ntheta, ug.T, dir_fwd_capacity(), dir_tol, dir_min, dplan);
        HostPlan hp;
        if (dirs) {  // per-direction sincos and adjoint entries; no per-ray items
            hp.sincos = dplan.sincos;
            hp.adj_pts = std::move(dplan.adj_pos);
            hp.adj_items = std::move(dplan.adj_items);
        } else {
            hp = build_plan(theta_h, n, ntheta, ug.T, table_capacity(), 1 << 30, tc_min_spr);
        }
        auto up = [&](const void *src, size_t bytes) -> void * {
            void *p = nullptr;
            CUDA_CHECK(cudaMallocAsync(&p, std::max<size_t>(bytes, 16), stream));
            geo_owned.push_back(p);
            geo_bytes += std::max<size_t>(bytes, 16);
            if (bytes) CUDA_CHECK(cudaMemcpyAsync(p, src, bytes, cudaMemcpyHostToDevice, stream));
            return p;
        };
        gd.sincos = (float2 *)up(hp.sincos.data(), hp.sincos.size() * sizeof(float2));
        gd.fwd_pts = (uint32_t *)up(hp.fwd_pts.data(), hp.fwd_pts.size() * 4);
        gd.fwd_items = (int4 *)up(hp.fwd_items.data(), hp.fwd_items.size() * sizeof(int4));
        gd.n_fwd_items = (int)hp.fwd_items.size();
        gd.fwd_tc_items = (int4 *)up(hp.fwd_tc_items.data(), hp.fwd_tc_items.size() * sizeof(int4));
        gd.n_fwd_tc_items = (int)hp.fwd_tc_items.size();
        gd.adj_pts = (uint32_t *)up(hp.adj_pts.data(), hp.adj_pts.size() * 4);
        gd.adj_items = (int4 *)up(hp.adj_items.data(), hp.adj_items.size() * sizeof(int4));
        gd.n_adj_items = (int)hp.adj_items.size();
        gd.n_adj_busy = 0;
        while (gd.n_adj_busy < gd.n_adj_items && hp.adj_items[gd.n_adj_busy].z > 0) ++gd.n_adj_busy;
        gd.split_tiles = (int *)up(hp.split_tiles.data(), hp.split_tiles.size() * 4);
        gd.n_split_tiles = (int)hp.split_tiles.size();
        gd.tc_scatter = tc_scatter;
        if (dirs) {
            gd.dirs = true;
            gd.ndir = dplan.ndir;
            gd.dray_start = (int *)up(dplan.ray_start.data(), dplan.ray_start.size() * sizeof(int));
            gd.drays = (uint32_t *)up(dplan.rays.data(), dplan.rays.size() * 4);
            gd.dtau = (float *)up(dplan.tau.data(), dplan.tau.size() * 4);
            gd.dfwd_pos = (uint32_t *)up(dplan.fwd_pos.data(), dplan.fwd_pos.size() * 4);
            gd.dfwd_items = (int4 *)up(dplan.fwd_items.data(), dplan.fwd_items.size() * sizeof(int4));
            gd.n_dfwd_items = (int)dplan.fwd_items.size();
            {  // the adjoint's E, E_perp per (slice, position) of one batch
                const size_t bytes = dir_mix_bytes(zb, dplan.ndir, n);
                void *p = nullptr;
                CUDA_CHECK(cudaMallocAsync(&p, bytes, stream));
                geo_owned.push_back(p);
                geo_bytes += bytes;
                gd.demix = (float4 *)p;
                gd.demix_slices = zb;
            }
        }
        std::vector<int> tab_base(1, 0);  // uploaded asynchronously: kept until the stream sync below
        std::vector<int4> tabs;
        if (tc_scatter) {
            void *p = nullptr;
            CUDA_CHECK(cudaMallocAsync(&p, std::max<size_t>(hp.adj_pts.size() * sizeof(AdjRec), 16), stream));
            geo_owned.push_back(p);
            geo_bytes += std::max<size_t>(hp.adj_pts.size() * sizeof(AdjRec), 16);
            gd.adj_recs = (AdjRec *)p;
            // tables of the busy items and the size of their ray segmentation
            const int cap = dirs ? dir_adj_table_capacity() : scatter_tc_table_capacity();
            long long words = 0;
            // a table holds whole rays (runs of equal theta), at most one MMA
            // batch of them (scatter_tc_batch_rays()) and at most cap entries;
            // on the direction path whole directions, at most dir_adj_table_dirs()
            const int max_rays = dirs ? dir_adj_table_dirs() : scatter_tc_batch_rays();
            for (int i = 0; i < gd.n_adj_busy; ++i) {
                const int4 it = hp.adj_items[i];
                const uint32_t *pts = hp.adj_pts.data() + it.y;
                int c0 = 0;
                while (c0 < it.z) {
                    int c1 = c0, nseg = 0;
                    while (c1 < it.z) {
                        int r = c1 + 1;  // end of the ray starting at c1
                        while (r < it.z && pts[r] / (uint32_t)n == pts[c1] / (uint32_t)n) ++r;
                        if (nseg > 0 && (nseg == max_rays || r - c0 > cap)) break;
                        if (r - c0 > cap) r = c0 + cap;  // a ray longer than a table is split
                        c1 = r;
                        ++nseg;
                    }
                    const int w = dirs ? dir_adj_info_words(nseg) : scatter_tc_info_words(nseg);
                    tabs.push_back(make_int4(it.y + c0, c1 - c0, (int)words, w));
                    words += w;
                    if (words > 2147483647LL) throw Error(RECTV_ERR_ARG, "rectv: adjoint plan too large");
                    c0 = c1;
                }
                tab_base.push_back((int)tabs.size());
            }
            gd.n_adj_tabs = (int)tabs.size();
            gd.adj_tabs = (int4 *)up(tabs.data(), tabs.size() * sizeof(int4));
            gd.adj_tab_base = (int *)up(tab_base.data(), tab_base.size() * sizeof(int));
            void *q = nullptr;
            CUDA_CHECK(cudaMallocAsync(&q, std::max<size_t>((size_t)words * 4, 16), stream));
            geo_owned.push_back(q);
            geo_bytes += std::max<size_t>((size_t)words * 4, 16);
            gd.adj_info = (uint32_t *)q;
        }
        if (gd.n_fwd_items > 2147483647 || gd.n_adj_items > 2147483647)
            throw Error(RECTV_ERR_ARG, "rectv: plan too large");

        // K'(theta, j) = ntheta/sqrt(m) sum_i phi_i(theta) conj(phi_i(t_j)),
        // t_j = j*ntheta/m: decphi/mulphi/recphi (kernels_operators.cuh:99-149)
        // phi_h == nullptr: the plain (static) Radon transform into time sample 0,
        // K'(theta, 0) = 1, K'(theta, j > 0) = 0 (filtered backprojection)
        std::vector<float2> kmat((size_t)ntheta * m, make_float2(0.f, 0.f));
        const double cphi = (double)ntheta / std::sqrt((double)m);
        if (!phi_h)
            for (int th = 0; th < ntheta; ++th) kmat[(size_t)th * m] = make_float2(1.f, 0.f);
        for (int th = 0; phi_h && th < ntheta; ++th)
            for (int j = 0; j < m; ++j) {
                const int tj = (int)(((long long)j * ntheta) / m);
                std::complex<double> acc(0.0, 0.0);
                for (int i = 0; i < m; ++i) {
                    const std::complex<double> a(phi_h[(size_t)i * 2 * ntheta + 2 * th],
                                                 phi_h[(size_t)i * 2 * ntheta + 2 * th + 1]);
                    const std::complex<double> b(phi_h[(size_t)i * 2 * ntheta + 2 * tj],
                                                 phi_h[(size_t)i * 2 * ntheta + 2 * tj + 1]);
                    acc += a * std::conj(b);
                }
                acc *= cphi;
                kmat[(size_t)th * m + j] = make_float2((float)acc.real(), (float)acc.imag());
            }
        gd.kmat = (float2 *)up(kmat.data(), kmat.size() * sizeof(float2));
        // set_center (radonusfft.cu:70-75, takeshift kernels_radonusfft.cuh:191-198)
        std::vector<float2> sf(n), sa(n);
        for (int k = 0; k < n; ++k) {
            const double cf = -((double)center - n / 2.0), ca = (double)center - n / 2.0;
            const double af = 2 * kPiUsfft * cf * (k - n / 2.0) / n;
            const double aa = 2 * kPiUsfft * ca * (k - n / 2.0) / n;
            sf[k] = make_float2((float)std::cos(af), (float)std::sin(af));
            sa[k] = make_float2((float)std::cos(aa), (float)std::sin(aa));
        }
        gd.shiftfwd = (float2 *)up(sf.data(), n * sizeof(float2));
        gd.shiftadj = (float2 *)up(sa.data(), n * sizeof(float2));
        // 1/phi of divphi (kernels_radonusfft.cuh:11), separable
        std::vector<float> dp(n);
        for (int x = 0; x < n; ++x) {
            const double d = (double)(x - n / 2);
            dp[x] = (float)std::exp((double)mu_us * d * d);
        }
        gd.deapod = (float *)up(dp.data(), n * sizeof(float));
        if (gd.tc_scatter) {
            if (gd.dirs) {
                launch_adj_records_dir(gd.adj_recs, gd, ug, stream);
                launch_adj_tabinfo_dir(gd, stream);
            } else {
                launch_adj_records(gd.adj_recs, gd, ug, stream);
                launch_adj_tabinfo(gd, stream);
            }
        }
        CUDA_CHECK(cudaStreamSynchronize(stream));  // host vectors go out of scope
        geo_theta.assign(theta_h, theta_h + ntheta);
        geo_phi.assign(phi_h, phi_h + nphi);
        geo_has_phi = phi_h != nullptr;
        geo_center = center;
        geo_tc_spr = tc_min_spr;
        geo_tc_scatter = tc_scatter;
        geo_dir_min = dir_min;
        geo_dir_tol = dir_tol;
        geo_valid = true;
        return true;
    }

    // ---- operators on one batch of zb slices ----
    // out = tau R_apr u  (residual: out = R_apr u - gb)
    void forward(const float *u, const float *gb, float *out, float tau, int residual) {
        forward_rows(u);
        CUFFT_CHECK(cufftExecC2C(p_rows_c2c, reinterpret_cast<cufftComplex *>(rows),
                                 reinterpret_cast<cufftComplex *>(rows), CUFFT_INVERSE));
        launch_finish_fwd(rows, gb, out, zb, tau, residual, ug, stream);
    }

    // the gathered row spectra of R_apr u (before the inverse row FFT) in rows
    void forward_rows(const float *u) {
        const int nimg = zb * m;
        if (pad_fft) {
            launch_pad_fft_fwd(u, spec, nimg, gd.deapod, fft_tw, fft_fwd_map, gd.err, ug, stream);
        } else {
            launch_deapod_pad(u, reinterpret_cast<float *>(spec), nimg, gd.deapod, ug, stream);
            for (int i = 0; i < nimg; i += img_per_fft) {
                cufftComplex *p = reinterpret_cast<cufftComplex *>(spec + (size_t)i * ug.img_fwd + ug.qoff);
                CUFFT_CHECK(cufftExecR2C(p_r2c2d, reinterpret_cast<cufftReal *>(p), p));
            }
        }
        launch_spec_halo(spec, nimg, ug, stream);
        launch_gather_fwd(spec, rows, zb, gd, ug, &spec_tmap, stream);
    }

    // u += tau R_apr^T h
    void adjoint(const float *h, float *u, float tau, const float *row_filter = nullptr) {
        launch_adj_prep(h, reinterpret_cast<float *>(rows), zb, ug, stream);
        CUFFT_CHECK(cufftExecR2C(p_rows_r2c, reinterpret_cast<cufftReal *>(rows),
                                 reinterpret_cast<cufftComplex *>(rows)));
        if (row_filter) launch_filter_rows(rows, row_filter, (long long)zb * ntheta, n, stream);
        adjoint_rows(rows, u, tau);
    }

    // u += tau R_apr^T of the row spectra rowsc [zb][ntheta][n/2+1]
    void adjoint_rows(const float2 *rowsc, float *u, float tau) {
        const int nimg = zb * m;
        if (gd.tc_scatter) {
            // Re IFFT2 of the scattered grids as a C2R of their Hermitian part,
            // which the tensor-core scatter adds into zeroed half planes
            const long long img_half = (long long)ug.P * ug.hpitch;
            // (the direction path clears them inside k_adj_mix)
            if (!gd.dirs) CUDA_CHECK(cudaMemsetAsync(spec, 0, sizeof(float2) * (size_t)nimg * img_half, stream));
            launch_scatter_adj(rowsc, spec, zb, gd, ug, stream);
            if (pad_fft) {
                launch_pad_fft_inv_accum(spec, u, zb, tau, gd.deapod, fft_tw, fft_inv_map, gd.err, ug, stream);
                return;
            }
            for (int i = 0; i < nimg; i += img_per_fft) {
                cufftComplex *p = reinterpret_cast<cufftComplex *>(spec + (size_t)i * img_half);
                CUFFT_CHECK(cufftExecC2R(p_c2r2d, p, reinterpret_cast<cufftReal *>(p)));
            }
            launch_crop_accum_real(reinterpret_cast<const float *>(spec), u, zb, tau, gd.deapod, ug, stream);
            return;
        }
        if (lay.img_spec < (long long)ug.P * ug.P)
            throw Error(RECTV_ERR_STATE, "rectv: spectra buffer sized for half planes, FP32 scatter needs full planes");
        launch_zero_split(spec, zb, gd, ug, stream);
        launch_scatter_adj(rowsc, spec, zb, gd, ug, stream);
        for (int i = 0; i < nimg; i += img_per_fft) {
            cufftComplex *p = reinterpret_cast<cufftComplex *>(spec + (size_t)i * ug.img_adj);
            CUFFT_CHECK(cufftExecC2C(p_c2c2d, p, p, CUFFT_INVERSE));
        }
        launch_crop_accum(spec, u, zb, tau, gd.deapod, ug, stream);
    }

    // ---- one outer ADMM iteration (rectv.cu:140-245 for all chunks) ----
    void enqueue_outer(int old) {
        const int a = (old + 1) % 3, b = (old + 2) % 3;
        int src = old;
        const int dpb = zb / nzp;  // chunks per batch
        for (int k = 0; k < titer; ++k) {
            const int dst = (k % 2 == 0) ? a : b;
            for (int bb = 0; bb < nbatch; ++bb) {
                const long long z0 = (long long)bb * zb;
                const int c0 = bb * dpb;
                if (fused_rows) {  // residual rows straight into the adjoint's row spectra
                    forward_rows(U[src] + z0 * slab);
                    launch_resid_rows(rows, gdata + z0 * ntheta * n, rows_adj, fft_tw_n, zb, ug, stream);
                } else {
                    forward(U[src] + z0 * slab, gdata + z0 * ntheta * n, h1, 1.0f, 1);
                }
                // first inner step: psi, mu in, w = mu - rho psi out; later steps: w in
                const int gmode = titer > 1 ? (k == 0 ? 1 : 2) : 0;
                launch_graddiv(U[src], U[old], U[dst], psi, mu, wdual, gmode, rho_d, c0, nchunks, tv, stream);
                if (fused_rows)
                    adjoint_rows(rows_adj, U[dst] + z0 * slab, -0.5f);
                else
                    adjoint(h1, U[dst] + z0 * slab, -0.5f);
            }
            src = dst;
        }
        for (int bb = 0; bb < nbatch; ++bb) {
            launch_shrink(U[src], U[old], psi, mu, rho_d, lambda0, bb * dpb, nchunks, tv,
                          partials + (size_t)3 * nparts_batch * bb, stream);
        }
        launch_reduce_rho(partials, nparts_batch * nbatch, stage1, rho_d, stats, iter_ctr, stats_cap, stream);
    }

    int next_cur(int old) const {
        if (titer == 0) return old;
        return (titer % 2 == 1) ? (old + 1) % 3 : (old + 2) % 3;
    }

    void launch_outer() {
        const int old = cur;
        if (use_graphs) {
            if (!graphs[old]) {
                cudaGraph_t g = nullptr;
                CUDA_CHECK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
                try {
                    enqueue_outer(old);
                } catch (...) {
                    cudaStreamEndCapture(stream, &g);
                    if (g) cudaGraphDestroy(g);
                    throw;
                }
                CUDA_CHECK(cudaStreamEndCapture(stream, &g));
                cudaGraphExec_t ge = nullptr;
                cudaError_t e = cudaGraphInstantiate(&ge, g, 0);
                cudaGraphDestroy(g);
                CUDA_CHECK(e);
                graphs[old] = ge;
            }
            CUDA_CHECK(cudaGraphLaunch(graphs[old], stream));
        } else {
            enqueue_outer(old);
        }
        cur = next_cur(old);
    }

    void setup(const float *theta_h, const float *phi_h, float center, float lambda0_, float lambda1_,
               int titer_, const float *init = nullptr, cudaMemcpyKind init_kind = cudaMemcpyHostToDevice) {
        check_live();
        if (titer_ < 0) throw Error(RECTV_ERR_ARG, "rectv: titer must be >= 0");
        if (!phi_h) throw Error(RECTV_ERR_ARG, "rectv: phi is required");
        const bool rebuilt = set_geometry(theta_h, phi_h, center);
        if (lay.iter_plans) ensure_plans();
        lambda0 = lambda0_;
        set_lambda1(lambda1_);
        titer = titer_;
        // graphs bake in the geometry, titer and the two lambdas
        if (rebuilt || titer != graph_titer || lambda0 != graph_lambda0 || lambda1 != graph_lambda1) {
            drop_graphs();
            graph_titer = titer;
            graph_lambda0 = lambda0;
            graph_lambda1 = lambda1;
        }
        // initial guess (zero, as rectv.cu:119-120, unless given) and ADMM state (rectv.cu:121-125)
        cur = 0;
        if (init)
            CUDA_CHECK(cudaMemcpyAsync(U[0], init, sizeof(float) * (size_t)nzc * slab, init_kind, stream));
        else
            CUDA_CHECK(cudaMemsetAsync(U[0], 0, sizeof(float) * (size_t)nzc * slab, stream));
        CUDA_CHECK(cudaMemsetAsync(psi, 0, sizeof(float) * (size_t)4 * nchunks * gp, stream));
        CUDA_CHECK(cudaMemsetAsync(mu, 0, sizeof(float) * (size_t)4 * nchunks * gp, stream));
        const float rho0 = 0.5f;
        CUDA_CHECK(cudaMemcpyAsync(rho_d, &rho0, sizeof(float), cudaMemcpyHostToDevice, stream));
        CUDA_CHECK(cudaStreamSynchronize(stream));
        iters_done = 0;
        h_rdiff.clear();
        h_rho.clear();
        h_r.clear();
        h_s.clear();
        session = true;
    }

    void ensure_stats(int cap) {
        if (cap <= stats_cap) return;
        drop_graphs();  // graphs hold the stats pointer
        if (stats) {
            cudaFreeAsync(stats, stream);
            owned.erase(std::find(owned.begin(), owned.end(), (void *)stats));
            dev_bytes -= sizeof(double) * (size_t)4 * stats_cap;
        }
        stats = alloc<double>((size_t)4 * cap);
        stats_cap = cap;
    }

    void report(int it, int niter_total, const double *row) {
        h_rdiff.push_back(row[0]);
        h_rho.push_back(row[1]);
        h_r.push_back(row[2]);
        h_s.push_back(row[3]);
        if (verbose) {
            std::fprintf(stderr, "iter (%d/%d), rdiff ||f(k+1)-f(k)||:%f \n", it, niter_total, row[0]);
            std::fflush(stderr);
        }
    }

    void iterate(int niter) {
        check_live();
        if (!session) throw Error(RECTV_ERR_STATE, "rectv: setup must precede iterate");
        if (niter < 0) throw Error(RECTV_ERR_ARG, "rectv: niter must be >= 0");
        if (niter == 0) return;
        ensure_stats(niter);
        if (stats_host_cap < niter) {
            if (stats_host) cudaFreeHost(stats_host);
            stats_host = nullptr;
            stats_host_cap = 0;
            CUDA_CHECK(cudaMallocHost(&stats_host, sizeof(double) * 4 * niter));
            stats_host_cap = niter;
        }
        CUDA_CHECK(cudaMemsetAsync(iter_ctr, 0, sizeof(int), stream));
        std::vector<cudaEvent_t> ev;
        if (verbose) {
            ev.resize(niter);
            for (auto &e : ev) CUDA_CHECK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        }
        int reported = 0;
        try {
            for (int it = 0; it < niter; ++it) {
                launch_outer();
                if (verbose) {
                    CUDA_CHECK(cudaMemcpyAsync(stats_host + 4 * it, stats + 4 * it, 4 * sizeof(double),
                                               cudaMemcpyDeviceToHost, stream));
                    CUDA_CHECK(cudaEventRecord(ev[it], stream));
                    // report the previous iteration while this one runs
                    while (reported < it) {
                        CUDA_CHECK(cudaEventSynchronize(ev[reported]));
                        report(iters_done + reported, niter, stats_host + 4 * reported);
                        ++reported;
                    }
                }
            }
            if (verbose) {
                while (reported < niter) {
                    CUDA_CHECK(cudaEventSynchronize(ev[reported]));
                    report(iters_done + reported, niter, stats_host + 4 * reported);
                    ++reported;
                }
            } else {
                CUDA_CHECK(cudaMemcpyAsync(stats_host, stats, 4 * sizeof(double) * niter, cudaMemcpyDeviceToHost,
                                           stream));
                CUDA_CHECK(cudaStreamSynchronize(stream));
                for (int it = 0; it < niter; ++it) {
                    h_rdiff.push_back(stats_host[4 * it]);
                    h_rho.push_back(stats_host[4 * it + 1]);
                    h_r.push_back(stats_host[4 * it + 2]);
                    h_s.push_back(stats_host[4 * it + 3]);
                }
            }
        } catch (...) {
            for (auto &e : ev) cudaEventDestroy(e);
            throw;
        }
        for (auto &e : ev) cudaEventDestroy(e);
        iters_done += niter;
        check_device_errors();
    }

    // Queues niter outer iterations on the handle's stream and returns
    // without waiting; their statistics stay on the device until
    // collect_history().  (The engine's asynchronous form of iterate().)
    void enqueue_iterations(int niter) {
        check_live();
        if (!session) throw Error(RECTV_ERR_STATE, "rectv: setup must precede iterate");
        if (niter < 0) throw Error(RECTV_ERR_ARG, "rectv: niter must be >= 0");
        pending = niter;
        if (niter == 0) return;
        ensure_stats(niter);
        CUDA_CHECK(cudaMemsetAsync(iter_ctr, 0, sizeof(int), stream));
        for (int it = 0; it < niter; ++it) launch_outer();
    }

    // After the stream has finished the queued iterations: appends their
    // statistics to the history (pageable host copy, no pinned buffer) and
    // raises if a kernel recorded an error.
    void collect_history() {
        if (pending > 0) {
            std::vector<double> row((size_t)4 * pending);
            CUDA_CHECK(cudaMemcpyAsync(row.data(), stats, sizeof(double) * row.size(), cudaMemcpyDeviceToHost, stream));
            CUDA_CHECK(cudaStreamSynchronize(stream));
            for (int it = 0; it < pending; ++it) {
                h_rdiff.push_back(row[4 * it]);
                h_rho.push_back(row[4 * it + 1]);
                h_r.push_back(row[4 * it + 2]);
                h_s.push_back(row[4 * it + 3]);
            }
            iters_done += pending;
        }
        pending = 0;
        check_device_errors();
    }

    // Waits for the stream and raises if a kernel recorded an error on the
    // device since the handle was created: a host/device plan disagreement
    // or a bounded TMA / tensor-core wait that gave up.
    void check_device_errors() {
        int errs = 0;
        CUDA_CHECK(cudaMemcpyAsync(&errs, gd.err, sizeof(int), cudaMemcpyDeviceToHost, stream));
        CUDA_CHECK(cudaStreamSynchronize(stream));
        if (errs)
            throw Error(RECTV_ERR_STATE,
                        "rectv: internal kernel error (plan/stencil mismatch or a TMA / tensor-core wait timed out)");
    }

    // ---- operator API helpers: any number of slices via zero-padded batches ----
    void op_forward(float *out, const float *u, int nslices, float tau) {
        ensure_plans();
        for (int z0 = 0; z0 < nslices; z0 += zb) {
            const int nb = std::min(zb, nslices - z0);
            const float *src = u + (size_t)z0 * slab;
            float *dst = out + (size_t)z0 * ntheta * n;
            if (nb == zb) {
                forward(src, nullptr, dst, tau, 0);
            } else {
                float *tmp = U[2];
                CUDA_CHECK(cudaMemsetAsync(tmp, 0, sizeof(float) * zb * slab, stream));
                CUDA_CHECK(cudaMemcpyAsync(tmp, src, sizeof(float) * nb * slab, cudaMemcpyDeviceToDevice, stream));
                forward(tmp, nullptr, h1, tau, 0);
                CUDA_CHECK(cudaMemcpyAsync(dst, h1, sizeof(float) * nb * ntheta * n, cudaMemcpyDeviceToDevice,
                                           stream));
            }
        }
    }

    void op_adjoint(float *u, const float *g, int nslices, float tau) {
        ensure_plans();
        for (int z0 = 0; z0 < nslices; z0 += zb) {
            const int nb = std::min(zb, nslices - z0);
            const float *src = g + (size_t)z0 * ntheta * n;
            float *dst = u + (size_t)z0 * slab;
            if (nb == zb) {
                adjoint(src, dst, tau);
            } else {
                CUDA_CHECK(cudaMemsetAsync(h1, 0, sizeof(float) * zb * ntheta * n, stream));
                CUDA_CHECK(cudaMemcpyAsync(h1, src, sizeof(float) * nb * ntheta * n, cudaMemcpyDeviceToDevice,
                                           stream));
                float *tmp = U[2];
                CUDA_CHECK(cudaMemsetAsync(tmp, 0, sizeof(float) * zb * slab, stream));
                adjoint(h1, tmp, 1.0f);
                launch_axpy(dst, tmp, tau, (long long)nb * slab);
            }
        }
    }

    void launch_axpy(float *y, const float *x, float a, long long count);

    // ---- filtered backprojection (static object), per slice ----
    // frec[z] = circ( pi/4 * R^T( applyfilter(g[z]) ) ): the USFFT adjoint with
    // the reference's ramp filter (kernels_radonusfft.cuh:173-189) on the
    // centred row spectrum and its circular mask (kernels_radonusfft.cuh:
    // 146-159, r = 0).  pi/4 makes R^T W R the identity on band-limited,
    // zero-mean objects for this operator's 1/sqrt(n ntheta) normalisation.
    void fbp(float *frec_h, const float *g_h, const float *theta_h, float center) {
        check_live();
        session = false;
        drop_graphs();
        ensure_plans();
        set_geometry(theta_h, nullptr, center);
        std::vector<float> w(n / 2 + 1);
        for (int k = 0; k <= n / 2; ++k) {
            const float rho = (float)(k - n / 2) / (float)n;
            w[k] = (rho == 0.f) ? 0.f : (float)(std::fabs((double)rho) * n * 4 * std::sin((double)rho) / rho);
        }
        float *w_d = nullptr;
        CUDA_CHECK(cudaMallocAsync(&w_d, w.size() * sizeof(float), stream));
        geo_owned.push_back(w_d);
        CUDA_CHECK(cudaMemcpyAsync(w_d, w.data(), w.size() * sizeof(float), cudaMemcpyHostToDevice, stream));
        const float scale = (float)(kPiUsfft / 4.0);
        float *tmp = U[2], *out = U[1];
        for (int z0 = 0; z0 < nz; z0 += zb) {
            const int nb = std::min(zb, nz - z0);
            CUDA_CHECK(cudaMemsetAsync(h1, 0, sizeof(float) * (size_t)zb * ntheta * n, stream));
            CUDA_CHECK(cudaMemcpyAsync(h1, g_h + (size_t)z0 * ntheta * n, sizeof(float) * (size_t)nb * ntheta * n,
                                       cudaMemcpyHostToDevice, stream));
            CUDA_CHECK(cudaMemsetAsync(tmp, 0, sizeof(float) * (size_t)zb * slab, stream));
            adjoint(h1, tmp, scale, w_d);
            launch_fbp_mask(tmp, out, nb, n, m, 0.f, stream);
            CUDA_CHECK(cudaMemcpyAsync(frec_h + (size_t)z0 * n * n, out, sizeof(float) * (size_t)nb * n * n,
                                       cudaMemcpyDeviceToHost, stream));
            CUDA_CHECK(cudaStreamSynchronize(stream));
        }
        free_geo();  // the FBP geometry is not the reconstruction's
    }

    // ---- instrumentation ----
    int jgroups() const { return (m + 15) / 16; }
    void launch_counts(int *kern, int *ffts) const {
        const int nimg = zb * m;
        const int f2 = img_per_fft > 0 ? (nimg + img_per_fft - 1) / img_per_fft : 0;
        const int ng = jgroups();
        // the padded-grid FFTs replace deapodise/pad (crop) and the 2D cuFFT
        // executions by a row and a column kernel each
        const bool own2d = pad_fft && gd.tc_scatter;
        // forward: [rows + columns | deapodise/pad], halo, zeroing of the k = 0
        // samples, per group of 16 time samples the tensor-core gather (8+ time
        // samples) and the direct one (items with few samples per ray), then the
        // fused residual rows or the forward epilogue
        const int gather_k =
            1 + ng * (gd.dirs ? (gd.n_dfwd_items > 0 ? 1 : 0)
                              : ((m >= 8 && gd.n_fwd_tc_items > 0) ? 1 : 0) + (gd.n_fwd_items > 0 ? 1 : 0));
        const int fwd_k = (pad_fft ? 2 : 1) + 1 + gather_k + 1;
        const int fwd_f = (pad_fft ? 0 : f2) + (fused_rows ? 0 : 1);
        // adjoint: [row preparation], the zeroing of split tiles (direct scatter),
        // one scatter per group, then [columns + rows | crop]
        const int adj_k = (fused_rows ? 0 : 1) + ((!gd.tc_scatter && gd.n_split_tiles > 0) ? 1 : 0) +
                          ng * (gd.dirs ? 2 : 1) +
                          (own2d ? 2 : 1);
        const int adj_f = (fused_rows ? 0 : 1) + (own2d ? 0 : f2);
        // per outer iteration: titer inner steps per batch (forward, graddiv,
        // adjoint), one shrink per batch, the two-stage rho reduction
        *kern = titer * nbatch * (fwd_k + 1 + adj_k) + nbatch + 2;
        *ffts = titer * nbatch * (fwd_f + adj_f);
    }

    void kernel_cost(int which, double *bytes, double *flops) const {
        const double P = 2.0 * n;
        const double npts = (double)ntheta * (n - 1) * zb;  // polar samples per launch
        const int dpb = zb / nzp;
        switch (which) {
            case 0:  // gather: half-plane spectra in, complex rows out
                *bytes = (double)zb * m * P * (P / 2 + 1) * 8.0 + (double)zb * ntheta * n * 8.0;
                *flops = npts * (81.0 * 2.0 * m * 2.0 + 8.0 * m + 18.0 * 4.0);
                break;
            case 1:  // scatter: half row spectra in; Hermitian half planes out (tensor-core path), else full planes
                *bytes = (double)zb * ntheta * (n / 2 + 1) * 8.0 +
                         (gd.tc_scatter ? (double)zb * m * P * (P / 2 + 1) * 8.0 : (double)zb * m * P * P * 8.0);
                *flops = npts * (81.0 * 2.0 * m * 2.0 + 8.0 * m + 18.0 * 4.0);
                break;
            case 2:  // graddiv after the first inner step: u in, u out, w in (psi and mu when titer = 1)
                *bytes = (double)zb * slab * 8.0 + (titer > 1 ? 1.0 : 2.0) * 4.0 * dpb * gp * 4.0;
                *flops = (double)zb * slab * 60.0;
                break;
            case 6:  // graddiv of the first inner step: u in, u out, psi and mu in, w out
                *bytes = (double)zb * slab * 8.0 + (titer > 1 ? 3.0 : 2.0) * 4.0 * dpb * gp * 4.0;
                *flops = (double)zb * slab * 60.0;
                break;
            case 3:  // shrink: u_cur, u_old in, mu in, psi and mu out
                *bytes = (double)zb * slab * 8.0 + 3.0 * 4.0 * dpb * gp * 4.0;
                *flops = (double)dpb * gp * 80.0;
                break;
            case 4:    // padded forward FFT: u in; half rows of the n centre rows out, in again; P rows out
            case 5: {  // padded inverse FFT: P rows in; n centre rows out, in again; u read and written
                const double nimg = (double)zb * m, hp = (double)n + 1.0;
                const double half_rows = (double)n * hp * 8.0;
                *bytes = which == 4 ? nimg * (4.0 * n * n + 2.0 * half_rows + P * hp * 8.0)
                                    : nimg * (P * hp * 8.0 + 2.0 * half_rows + 8.0 * n * n);
                // 5 P log2 P flops per complex P-point transform: n/2 row pairs and n+1 columns
                *flops = nimg * (n / 2 + n + 1) * 5.0 * P * std::log2(P);
                break;
            }
            default:
                throw Error(RECTV_ERR_ARG, "rectv_kernel_cost: unknown kernel id");
        }
    }

    void launch_kernel(int which, int reps) {
        check_live();
        if (!session) throw Error(RECTV_ERR_STATE, "rectv_launch_kernel: needs a set-up session");
        if (which < 0 || which > 6) throw Error(RECTV_ERR_ARG, "rectv_launch_kernel: unknown kernel id");
        if ((which == 4 || which == 5) && !pad_fft)
            throw Error(RECTV_ERR_ARG, "rectv_launch_kernel: no padded-grid FFT at this size");
        for (int r = 0; r < reps; ++r) {
            switch (which) {
                case 0: launch_gather_fwd(spec, rows, zb, gd, ug, &spec_tmap, stream); break;
                case 1: launch_scatter_adj(fused_rows ? rows_adj : rows, spec, zb, gd, ug, stream); break;
                case 2:  // the inner steps after the first (w = mu - rho psi as stored by the last iteration)
                    launch_graddiv(U[cur], U[cur], U[(cur + 1) % 3], psi, mu, wdual, titer > 1 ? 2 : 0, rho_d, 0,
                                   nchunks, tv, stream);
                    break;
                case 3:  // overwrites the session's dual variables
                    launch_shrink(U[cur], U[cur], psi, mu, rho_d, lambda0, 0, nchunks, tv, partials, stream);
                    break;
                case 4:  // padded-grid forward FFT of the batch (rows + columns)
                    launch_pad_fft_fwd(U[cur], spec, zb * m, gd.deapod, fft_tw, fft_fwd_map, gd.err, ug, stream);
                    break;
                case 6:  // the first inner step (psi, mu in; stores w = mu - rho psi, unchanged values)
                    launch_graddiv(U[cur], U[cur], U[(cur + 1) % 3], psi, mu, wdual, titer > 1 ? 1 : 0, rho_d, 0,
                                   nchunks, tv, stream);
                    break;
                case 5:  // padded-grid inverse FFT (columns + rows), added into the scratch iterate
                    launch_pad_fft_inv_accum(spec, U[(cur + 1) % 3], zb, 0.f, gd.deapod, fft_tw, fft_inv_map, gd.err,
                                             ug, stream);
                    break;
                default: throw Error(RECTV_ERR_ARG, "rectv_launch_kernel: unknown kernel id");
            }
        }
    }

    void check_adjoints(double *res, const float *g_h, const float *theta_h, const float *phi_h,
                        float lambda1_, float center) {
        check_live();
        if (nz != nzp)
            throw Error(RECTV_ERR_ARG, "rectv: check_adjoints needs nz == nzp (one chunk), as in rectv.cu:258");
        session = false;
        drop_graphs();
        ensure_plans();
        set_geometry(theta_h, phi_h, center);
        set_lambda1(lambda1_);
        CUDA_CHECK(cudaMemcpyAsync(gdata, g_h, sizeof(float) * (size_t)nz * ntheta * n, cudaMemcpyHostToDevice,
                                   stream));
        float *f = U[0], *fn = U[1];
        CUDA_CHECK(cudaMemsetAsync(f, 0, sizeof(float) * (size_t)nzc * slab, stream));
        CUDA_CHECK(cudaMemsetAsync(fn, 0, sizeof(float) * (size_t)nzc * slab, stream));
        CUDA_CHECK(cudaMemsetAsync(dot_out, 0, sizeof(double) * 8, stream));
        // rectv.cu:266-275
        adjoint(gdata, f, 1.0f);
        forward(f, nullptr, h1, 1.0f, 0);
        const long long nf = (long long)nzc * slab, ng = (long long)nz * ntheta * n;
        launch_dot(f, f, nf, dot_part, dot_parts(), dot_out + 0, stream);
        launch_dot(gdata, h1, ng, dot_part, dot_parts(), dot_out + 1, stream);
        launch_dot(h1, h1, ng, dot_part, dot_parts(), dot_out + 2, stream);
        // rectv.cu:278-288 (gradient into the spectrum scratch, float4 layout)
        float *h2 = reinterpret_cast<float *>(spec);
        TvGeo t1 = tv;
        t1.nchunks = 1;
        launch_gradient_ref(f, 0, h2, 0, 0, t1, stream);
        launch_divergent_ref(fn, h2, 1.0f, t1, stream);
        launch_dot(f, fn, nf, dot_part, dot_parts(), dot_out + 3, stream);
        const long long npts = (long long)(n + 1) * (n + 1) * (m + 1) * (nz + 1);
        launch_dot(h2, h2, npts, dot_part, dot_parts(), dot_out + 4, stream);
        launch_dot(fn, fn, nf, dot_part, dot_parts(), dot_out + 5, stream);
        double r[8];
        CUDA_CHECK(cudaMemcpyAsync(r, dot_out, sizeof(double) * 8, cudaMemcpyDeviceToHost, stream));
        CUDA_CHECK(cudaStreamSynchronize(stream));
        for (int i = 0; i < 6; ++i) res[i] += r[i];
    }
};

// Launch shapes chosen by the autotuner (engine.cu): slices per block of the
// tensor-core gather and persistent blocks of the tensor-core scatter (0: one
// per SM), with the measured times of the chosen shapes.
struct Tune {
    int zper = 64;
    int sc_grid = 0;
    double gather_ms = 0, scatter_ms = 0;
};

// Times the candidate launch shapes on a handle with a set-up session,
// applies the fastest (dropping captured graphs) and returns them; cached per
// (device, n, ntheta, m, slices per launch) unless force.
Tune autotune(Handle &h, bool force);

}  // namespace rectv
