// Data ingest on the GPU: flat/dark-field normalisation, -log and the
// projection -> sinogram transpose that turns detector frames into the
// solver's input g[z][theta][s] (examples/tao/tao.py:34-41 of the reference:
//   data = -log((data - mean(dark)) / (1e-3 + mean(flat) - mean(dark))).swapaxes(0, 1)).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "rectv_gb300.h"
#include "rectv_internal.cuh"

namespace rectv {

namespace {

template <class T>
__device__ __forceinline__ float as_float(T v) {
    return (float)v;
}

// mean over frames of a [nframes][nz*n] stack -> [nz*n]
template <class T>
__global__ void k_frame_mean(const T *__restrict__ frames, int nframes, long long plane, float *__restrict__ out) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= plane) return;
    float acc = 0.f;
    for (int f = 0; f < nframes; ++f) acc += as_float(frames[(long long)f * plane + i]);
    out[i] = nframes > 0 ? acc / (float)nframes : 0.f;
}

// out[z][theta][x] = -log((data[theta][z][x] - dark[z][x]) / (1e-3 + flat[z][x] - dark[z][x]))
template <class T>
__global__ void k_normalize_transpose(const T *__restrict__ data, const float *__restrict__ dark,
                                      const float *__restrict__ flat, float *__restrict__ out, int ntheta,
                                      int nz, int n) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int th = blockIdx.y;
    const int z = blockIdx.z;
    if (x >= n) return;
    const long long zi = (long long)z * n + x;
    const float d = dark[zi];
    const float v = (as_float(data[((long long)th * nz + z) * n + x]) - d) / (1e-3f + flat[zi] - d);
    out[((long long)z * ntheta + th) * n + x] = -logf(v);
}

template <class T>
void preprocess_t(float *out, const void *data, const void *dark, const void *flat, int ntheta, int nz, int n,
                  int ndark, int nflat) {
    const size_t plane = (size_t)nz * n;
    const size_t nd = (size_t)ntheta * plane;
    T *d_data = nullptr, *d_dark = nullptr, *d_flat = nullptr;
    float *d_out = nullptr, *d_means = nullptr;
    cudaStream_t s = nullptr;
    auto cleanup = [&]() {
        if (s) cudaStreamDestroy(s);
        cudaFree(d_data);
        cudaFree(d_dark);
        cudaFree(d_flat);
        cudaFree(d_out);
        cudaFree(d_means);
    };
    try {
        CUDA_CHECK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
        CUDA_CHECK(cudaMalloc(&d_data, nd * sizeof(T)));
        CUDA_CHECK(cudaMalloc(&d_dark, std::max<size_t>(1, (size_t)ndark * plane) * sizeof(T)));
        CUDA_CHECK(cudaMalloc(&d_flat, std::max<size_t>(1, (size_t)nflat * plane) * sizeof(T)));
        CUDA_CHECK(cudaMalloc(&d_out, nd * sizeof(float)));
        CUDA_CHECK(cudaMalloc(&d_means, 2 * plane * sizeof(float)));
        CUDA_CHECK(cudaMemcpyAsync(d_data, data, nd * sizeof(T), cudaMemcpyHostToDevice, s));
        if (ndark) CUDA_CHECK(cudaMemcpyAsync(d_dark, dark, (size_t)ndark * plane * sizeof(T), cudaMemcpyHostToDevice, s));
        if (nflat) CUDA_CHECK(cudaMemcpyAsync(d_flat, flat, (size_t)nflat * plane * sizeof(T), cudaMemcpyHostToDevice, s));
        const unsigned gb = (unsigned)((plane + 255) / 256);
        k_frame_mean<T><<<gb, 256, 0, s>>>(d_dark, ndark, (long long)plane, d_means);
        LAUNCH_CHECK("k_frame_mean");
        k_frame_mean<T><<<gb, 256, 0, s>>>(d_flat, nflat, (long long)plane, d_means + plane);
        LAUNCH_CHECK("k_frame_mean");
        dim3 gs((n + 127) / 128, ntheta, nz);
        k_normalize_transpose<T><<<gs, 128, 0, s>>>(d_data, d_means, d_means + plane, d_out, ntheta, nz, n);
        LAUNCH_CHECK("k_normalize_transpose");
        CUDA_CHECK(cudaMemcpyAsync(out, d_out, nd * sizeof(float), cudaMemcpyDeviceToHost, s));
        CUDA_CHECK(cudaStreamSynchronize(s));
    } catch (...) {
        cleanup();
        throw;
    }
    cleanup();
}

}  // namespace

void preprocess(float *out, const void *data, const void *dark, const void *flat, int dtype, int ntheta, int nz,
                int n, int ndark, int nflat) {
    if (!out || !data || ntheta < 1 || nz < 1 || n < 1 || ndark < 0 || nflat < 0 || (ndark && !dark) ||
        (nflat && !flat))
        throw Error(RECTV_ERR_ARG, "rectv_preprocess: bad arguments");
    switch (dtype) {
        case RECTV_DTYPE_F32: preprocess_t<float>(out, data, dark, flat, ntheta, nz, n, ndark, nflat); break;
        case RECTV_DTYPE_U16: preprocess_t<uint16_t>(out, data, dark, flat, ntheta, nz, n, ndark, nflat); break;
        default: throw Error(RECTV_ERR_ARG, "rectv_preprocess: dtype must be RECTV_DTYPE_F32 or RECTV_DTYPE_U16");
    }
}

}  // namespace rectv

namespace rectv {

// ---------------------------------------------------------------------------
// Filtered backprojection helpers.  applyfilter (kernels_radonusfft.cuh:
// 173-189, never launched by the reference) weights the centred row spectrum
// by w(rho) = |rho| n 4 sin(rho)/rho, rho = (k - n/2)/n, w(0) = 0; circ
// (kernels_radonusfft.cuh:146-159) keeps 4x^2 + 4y^2 < 1 - r.
// ---------------------------------------------------------------------------
__global__ void k_filter_rows(float2 *__restrict__ rowsc, const float *__restrict__ w, long long nrows, int hn) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= nrows * hn) return;
    const int k = (int)(i % hn);
    const float c = w[k];
    float2 v = rowsc[i];
    rowsc[i] = make_float2(v.x * c, v.y * c);
}

void launch_filter_rows(float2 *rowsc, const float *w, long long nrows, int n, cudaStream_t s) {
    const int hn = n / 2 + 1;
    const long long total = nrows * hn;
    k_filter_rows<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(rowsc, w, nrows, hn);
    LAUNCH_CHECK("k_filter_rows");
}

// out[z][y][x] = circ mask * u[z][0][y][x]  (time sample 0 of a [z][m][n][n] volume)
__global__ void k_fbp_mask(const float *__restrict__ u, float *__restrict__ out, int n, int m, float r) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    const long long z = blockIdx.z;
    if (x >= n) return;
    const float xf = (x - n / 2) / (float)n, yf = (y - n / 2) / (float)n;
    const bool in = (4 * xf * xf + 4 * yf * yf) < 1 - r;
    out[(z * n + y) * n + x] = in ? u[((z * m) * n + y) * (long long)n + x] : 0.f;
}

void launch_fbp_mask(const float *u, float *out, int nslices, int n, int m, float r, cudaStream_t s) {
    dim3 gs((n + 127) / 128, n, nslices);
    k_fbp_mask<<<gs, 128, 0, s>>>(u, out, n, m, r);
    LAUNCH_CHECK("k_fbp_mask");
}

}  // namespace rectv
