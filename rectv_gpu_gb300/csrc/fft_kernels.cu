// Two-dimensional FFTs of the USFFT operators for P = 2n a power of two
// (256 <= P <= 2048), written for the zero padding of the reference's grids.
//
// The reference pads the deapodised n x n image into the centre of a P x P
// grid, modulates it by (-1)^(X+Y) and runs a P x P FFT (divphi, fftshift and
// the cuFFT 2D plan, radonusfft.cu:85-90, kernels_radonusfft.cuh:4-38); the
// adjoint runs the inverse FFT and crops the centre (radonusfft.cu:127-132).
// Three quarters of the forward input and of the adjoint output are padding,
// so the passes here touch only what is not:
//
//  forward  rows    n/2 row pairs per image: the pair's two deapodised real
//                   rows are one complex P-point FFT (a + i b, split after the
//                   transform), input read straight from the volume; writes
//                   the n+1 half-plane columns of rows [n/2, 3n/2)
//           columns n+1 columns of P points whose input rows outside
//                   [n/2, 3n/2) are zero (not read); writes all P rows
//  adjoint  columns n+1 inverse P-point FFTs of the Hermitian half planes;
//                   writes only rows [n/2, 3n/2) (in place)
//           rows    n/2 row pairs: the Hermitian extension of two half rows
//                   as one complex inverse FFT (Re -> first row, Im -> second),
//                   only the n centre outputs, deapodised and added into u
//
// The same transform core also runs the n-point row transforms between the
// gather and the scatter (k_resid_rows: inverse row FFT, residual, fftshift
// and the adjoint's row R2C in one pass, n a power of two in [256, 1024]).
//
// Every transform is P = 16 x 16 x R3 points (R3 = P/256) computed by P/16
// threads holding 16 values each: a 16-point DFT in registers, twiddles,
// exchange through shared memory, a 16-point DFT, twiddles, exchange, and
// R3-point DFTs.  Twiddles come from a table evaluated in double precision on
// the host, laid out so that the lanes of a warp read consecutive entries:
// [k2][n1] = exp(-2 pi i n1 k2 / P) for stage 1, then [j2][m1] =
// exp(-2 pi i 16 m1 j2 / P) for stage 2.  Results equal cuFFT's to FP32
// rounding.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "rectv_internal.cuh"
#include "tcgen05.cuh"

namespace rectv {

namespace {

__device__ __forceinline__ float2 operator+(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 operator-(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul_(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 conj_(float2 a) { return make_float2(a.x, -a.y); }

// a * exp(DIR * i pi / 2): DIR = -1 (forward) multiplies by -i, DIR = +1 by +i
template <int DIR>
__device__ __forceinline__ float2 rot4(float2 a) {
    return DIR < 0 ? make_float2(a.y, -a.x) : make_float2(-a.y, a.x);
}

// a * exp(DIR * 2 pi i e / 16) for a compile-time e in [0, 16)
template <int E, int DIR>
__device__ __forceinline__ float2 tw16(float2 a) {
    constexpr int e = E & 15;
    constexpr float C1 = 0.92387953251128674f;  // cos(pi/8)
    constexpr float S1 = 0.38268343236508977f;  // sin(pi/8)
    constexpr float R2 = 0.70710678118654752f;  // cos(pi/4)
    constexpr float cs[16] = {1.f, C1, R2, S1, 0.f, -S1, -R2, -C1, -1.f, -C1, -R2, -S1, 0.f, S1, R2, C1};
    constexpr float sn[16] = {0.f, S1, R2, C1, 1.f, C1, R2, S1, 0.f, -S1, -R2, -C1, -1.f, -C1, -R2, -S1};
    if constexpr (e == 0) {
        return a;
    } else if constexpr (e == 4) {
        return rot4<DIR>(a);
    } else if constexpr (e == 8) {
        return make_float2(-a.x, -a.y);
    } else if constexpr (e == 12) {
        return rot4<-DIR>(a);
    } else {
        constexpr float c = cs[e], s = DIR * sn[e];
        return make_float2(a.x * c - a.y * s, a.x * s + a.y * c);
    }
}

template <int DIR>
__device__ __forceinline__ void dft2(float2 &x0, float2 &x1) {
    const float2 s = x0 + x1, d = x0 - x1;
    x0 = s;
    x1 = d;
}

template <int DIR>
__device__ __forceinline__ void dft4(float2 &x0, float2 &x1, float2 &x2, float2 &x3) {
    const float2 s02 = x0 + x2, d02 = x0 - x2, s13 = x1 + x3, d13 = rot4<DIR>(x1 - x3);
    x0 = s02 + s13;
    x2 = s02 - s13;
    x1 = d02 + d13;
    x3 = d02 - d13;
}

// in place, natural order in and out: v[k] = sum_r v[r] exp(DIR 2 pi i r k / 8)
template <int DIR>
__device__ __forceinline__ void dft8(float2 *v) {
    // r = 2a + b, k = c + 4d
    dft4<DIR>(v[0], v[2], v[4], v[6]);  // b = 0 -> y0[c] at v[0], v[2], v[4], v[6]
    dft4<DIR>(v[1], v[3], v[5], v[7]);  // b = 1
    v[3] = tw16<2, DIR>(v[3]);          // omega8^c = omega16^(2c)
    v[5] = tw16<4, DIR>(v[5]);
    v[7] = tw16<6, DIR>(v[7]);
    float2 o[8];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        o[c] = v[2 * c] + v[2 * c + 1];
        o[c + 4] = v[2 * c] - v[2 * c + 1];
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = o[i];
}

// in place, natural order in and out: v[k] = sum_r v[r] exp(DIR 2 pi i r k / 16)
template <int DIR>
__device__ __forceinline__ void dft16(float2 *v) {
    // r = 4a + b, k = c + 4d: DFT4 over a for each b, twiddle omega16^(bc), DFT4 over b
#pragma unroll
    for (int b = 0; b < 4; ++b) dft4<DIR>(v[b], v[4 + b], v[8 + b], v[12 + b]);  // y[b][c] at v[4c + b]
    v[4 * 1 + 1] = tw16<1, DIR>(v[5]);
    v[4 * 1 + 2] = tw16<2, DIR>(v[6]);
    v[4 * 1 + 3] = tw16<3, DIR>(v[7]);
    v[4 * 2 + 1] = tw16<2, DIR>(v[9]);
    v[4 * 2 + 2] = tw16<4, DIR>(v[10]);
    v[4 * 2 + 3] = tw16<6, DIR>(v[11]);
    v[4 * 3 + 1] = tw16<3, DIR>(v[13]);
    v[4 * 3 + 2] = tw16<6, DIR>(v[14]);
    v[4 * 3 + 3] = tw16<9, DIR>(v[15]);
#pragma unroll
    for (int c = 0; c < 4; ++c) dft4<DIR>(v[4 * c], v[4 * c + 1], v[4 * c + 2], v[4 * c + 3]);  // over b
    // V[c + 4d] sits at v[4c + d]: transpose the 4x4 index
    float2 o[16];
#pragma unroll
    for (int c = 0; c < 4; ++c)
#pragma unroll
        for (int d = 0; d < 4; ++d) o[c + 4 * d] = v[4 * c + d];
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = o[i];
}

template <int R, int DIR>
__device__ __forceinline__ void dftR(float2 *v) {
    if constexpr (R == 2) dft2<DIR>(v[0], v[1]);
    if constexpr (R == 4) dft4<DIR>(v[0], v[1], v[2], v[3]);
    if constexpr (R == 8) dft8<DIR>(v);
    if constexpr (R == 16) dft16<DIR>(v);
}

__device__ __forceinline__ float2 twiddle(const float2 *__restrict__ tw, int e, int dir) {
    const float2 w = __ldg(tw + e);
    return dir < 0 ? w : make_float2(w.x, -w.y);
}

// Shared-memory layouts of one transform's values at the two exchanges.
//  INTERLEAVED (column kernels, thread = c + C t): element i of transform c
//    at i*C + c; stage-2 output of pair p, m1 at p*Q + m1 (Q = R3+1 odd).
//  regions (row kernels, thread = t + (P/16) c): element i of transform c at
//    c*S + i; stage-2 output at p*R3 + ((m1 + p/(16/R3)) mod R3).
// Both make the exchanges free of bank conflicts for P >= 1024 (at P = 512
// one exchange of the column kernels keeps a two-way conflict).
template <int N, bool INTERLEAVED, int C>
struct FftLayout {
    static constexpr int N1 = N / 16;
    static constexpr int R3 = N / 256;
    static constexpr int P1 = N1 + R3;
    static constexpr int Q = INTERLEAVED ? (R3 == 1 ? 1 : R3 + 1) : R3;
    static constexpr int S1 = 16 * P1;
    static constexpr int S2 = 256 * Q;
    static constexpr int S = (S1 > S2 ? S1 : S2) > N ? (S1 > S2 ? S1 : S2) : N;  // elements per transform
    __device__ static __forceinline__ int a1(int c, int i) { return INTERLEAVED ? i * C + c : c * S + i; }
    __device__ static __forceinline__ int a2(int c, int p, int m1) {
        if constexpr (INTERLEAVED) {
            return (p * Q + m1) * C + c;
        } else {
            constexpr int G = (R3 >= 16) ? 1 : 16 / R3;
            return c * S + p * R3 + ((R3 == 1) ? 0 : ((m1 + p / G) & (R3 - 1)));
        }
    }
};

// One P-point FFT per transform c; thread t of the transform enters with
// v[r] = x[t + N1 r] (r < 16) and leaves with v[q R3 + j1] = X[t + N1 q +
// 256 j1] (q < 16/R3, j1 < R3).  All threads of the block must call it.
template <int N, int DIR, class L>
__device__ __forceinline__ void fft_core(float2 *v, float2 *sh, int c, int t, const float2 *__restrict__ tw) {
    constexpr int N1 = L::N1, R3 = L::R3;
    // stage 1: 16-point DFT over n2 of x[n1 + N1 n2], twiddle omega_N^(n1 k2)
    dft16<DIR>(v);
#pragma unroll
    for (int k2 = 1; k2 < 16; ++k2) v[k2] = cmul_(v[k2], twiddle(tw, k2 * N1 + t, DIR));
#pragma unroll
    for (int k2 = 0; k2 < 16; ++k2) sh[L::a1(c, k2 * L::P1 + t)] = v[k2];
    __syncthreads();
    // stage 2: thread (k2, m1), 16-point DFT over m2 of y[k2][m1 + R3 m2]
    const int k2 = t / R3, m1 = t - k2 * R3;
#pragma unroll
    for (int m2 = 0; m2 < 16; ++m2) v[m2] = sh[L::a1(c, k2 * L::P1 + m1 + R3 * m2)];
    __syncthreads();
    dft16<DIR>(v);
#pragma unroll
    for (int j2 = 1; j2 < 16; ++j2) v[j2] = cmul_(v[j2], twiddle(tw, N + j2 * R3 + m1, DIR));
#pragma unroll
    for (int j2 = 0; j2 < 16; ++j2) sh[L::a2(c, k2 + 16 * j2, m1)] = v[j2];
    __syncthreads();
    // stage 3: R3-point DFTs over m1 for the pairs p = t + N1 q
#pragma unroll
    for (int q = 0; q < 16 / R3; ++q)
#pragma unroll
        for (int i = 0; i < R3; ++i) v[q * R3 + i] = sh[L::a2(c, t + N1 * q, i)];
    if constexpr (R3 > 1) {
#pragma unroll
        for (int q = 0; q < 16 / R3; ++q) dftR<R3, DIR>(v + q * R3);
    }
}

constexpr int kRowThreads = 512;  // threads per block of the row kernels
constexpr int kColC = 4;          // columns per block of the column kernels (32-byte row runs, two blocks per SM)

// ---------------------------------------------------------------------------
// Forward rows: deapodise, pad and modulate two rows of u (rows 2 pr, 2 pr+1
// of image img), FFT as a + i b, split into the two half spectra and store
// them at rows Y = y + n/2 of the halo-padded forward spectra, columns 0..n.
// ---------------------------------------------------------------------------
template <int N>
__global__ void __launch_bounds__(kRowThreads, 2)
    k_fft_rows_fwd(const float *__restrict__ u, float2 *__restrict__ spec, const float *__restrict__ dp,
                   const float2 *__restrict__ tw, UsGeo g, float inv4n2) {
    constexpr int N1 = N / 16, RP = kRowThreads / N1;
    using L = FftLayout<N, false, RP>;
    extern __shared__ float2 fft_sh[];
    const int n = N / 2;
    const int t = threadIdx.x % N1, c = threadIdx.x / N1;
    const int pr = blockIdx.x * RP + c;  // row pair
    const long long img = blockIdx.y;
    const bool ok = pr < n / 2;
    const int ya = 2 * pr, yb = ya + 1;
    float2 v[16];
    {
        const float *ua = u + (img * n + (ok ? ya : 0)) * (long long)n;
        const float *ub = ua + n;
        const int Ya = ya + n / 2;
        const float sa = ok ? ((Ya & 1) ? -dp[ya] : dp[ya]) * inv4n2 : 0.f;
        const float sb = ok ? ((Ya & 1) ? dp[yb] : -dp[yb]) * inv4n2 : 0.f;
#pragma unroll
        for (int r = 0; r < 16; ++r) {
            v[r] = make_float2(0.f, 0.f);
            if (r >= 4 && r < 12) {  // X = t + N1 r in [n/2, 3n/2)
                const int x = t + N1 * (r - 4), X = x + n / 2;
                const float w = (X & 1) ? -__ldg(dp + x) : __ldg(dp + x);
                v[r] = make_float2(__ldg(ua + x) * w * sa, __ldg(ub + x) * w * sb);
            }
        }
    }
    fft_core<N, -1, L>(v, fft_sh, c, t, tw);
    // Z in natural order, then A(k) = (Z(k) + conj Z(-k))/2, B(k) = (Z(k) - conj Z(-k))/(2i)
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 16 / L::R3; ++q)
#pragma unroll
        for (int j1 = 0; j1 < L::R3; ++j1) fft_sh[c * L::S + t + N1 * q + 256 * j1] = v[q * L::R3 + j1];
    __syncthreads();
    if (!ok) return;
    float2 *ra = spec + img * g.img_fwd + g.qoff + (long long)(ya + n / 2) * g.qp;
    float2 *rb = ra + g.qp;
    for (int k = t; k <= n; k += N1) {
        const float2 zk = fft_sh[c * L::S + k], zm = fft_sh[c * L::S + ((N - k) & (N - 1))];
        ra[k] = make_float2(0.5f * (zk.x + zm.x), 0.5f * (zk.y - zm.y));
        rb[k] = make_float2(0.5f * (zk.y + zm.y), 0.5f * (zm.x - zk.x));
    }
}

// TMA tile copies of the column kernels: boxes of 4 columns (8 floats) x BR
// rows of one image, landing in shared memory as [row][column].
__device__ __forceinline__ void tma_load3(void *dst, const CUtensorMap *map, int x, int y, int z, void *bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];\n" ::"r"(tc::smem_addr(dst)),
        "l"((unsigned long long)map), "r"(x), "r"(y), "r"(z), "r"(tc::smem_addr(bar))
        : "memory");
}
__device__ __forceinline__ void tma_store3(const CUtensorMap *map, int x, int y, int z, const void *src) {
    asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.tile.bulk_group [%0, {%1, %2, %3}], [%4];\n" ::"l"(
                     (unsigned long long)map),
                 "r"(x), "r"(y), "r"(z), "r"(tc::smem_addr(src))
                 : "memory");
}
__device__ __forceinline__ void tma_store_wait_read() {
    asm volatile("cp.async.bulk.wait_group.read 0;\n" ::: "memory");
}
__device__ __forceinline__ void mbar_expect(void *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(tc::smem_addr(bar)), "r"(bytes)
                 : "memory");
}


// ---------------------------------------------------------------------------
// Column passes.  Persistent blocks (one per SM) take tiles of 4 columns of
// one image round-robin, column groups fastest; the tile after the current
// one is loaded by TMA into the second landing buffer while the current one
// is transformed, and each output tile leaves by TMA stores from the exchange
// buffer, which the next tile reuses once those stores have read it.
//
// Forward: columns kx .. kx+3 of the row pass output (rows [n/2, 3n/2); the
// others are zero and not read), P-point FFT, all P rows written back in
// place (window coordinates of the halo-padded spectra: x = 2 (kHalo + kx)
// floats, y = kHalo + row; columns past n are halo cells, rewritten by the
// halo pass afterwards).
// Inverse: inverse P-point FFT of columns kx .. kx+3 of the Hermitian half
// planes [img][P][hpitch]; only rows [n/2, 3n/2) are written back (columns
// past the row pitch read as zeros and are not stored).
// ---------------------------------------------------------------------------
template <int N, int C, int DIR>
struct ColPass {
    static constexpr int n = N / 2;
    static constexpr int BR = n < 256 ? n : 256;                // rows per TMA box
    static constexpr int IN_ROWS = DIR < 0 ? n : N;              // rows loaded per tile
    static constexpr int OUT_ROWS = DIR < 0 ? N : n;             // rows stored per tile
    static constexpr int IN_Y0 = DIR < 0 ? kHalo + n / 2 : 0;    // first loaded row (map coordinates)
    static constexpr int OUT_Y0 = DIR < 0 ? kHalo : n / 2;       // first stored row
    static constexpr int XOFF = DIR < 0 ? kHalo : 0;             // column offset of the map window
    using L = FftLayout<N, true, C>;
    static constexpr size_t EX = (size_t)L::S * C > (size_t)OUT_ROWS * C ? (size_t)L::S * C : (size_t)OUT_ROWS * C;
    static constexpr size_t LAND = (size_t)IN_ROWS * C;          // float2 per landing buffer
    static constexpr size_t SMEM = sizeof(float2) * (EX + 2 * LAND);
};

template <int N, int C, int DIR>
__global__ void __launch_bounds__(C *(N / 16), 1)
    k_fft_cols(const __grid_constant__ CUtensorMap tmap, const float2 *__restrict__ tw, int ngroups, int ntiles,
               int *__restrict__ err) {
    using CP = ColPass<N, C, DIR>;
    using L = typename CP::L;
    constexpr int N1 = N / 16, n = N / 2, BR = CP::BR;
    extern __shared__ __align__(1024) float2 fft_sh[];
    float2 *ex = fft_sh;  // exchange buffer / output tile; landing buffers follow it
    __shared__ uint64_t bar[2];
    const int c = threadIdx.x % C, t = threadIdx.x / C;
    if (threadIdx.x == 0) {
        tc::mbar_init(&bar[0], 1);
        tc::mbar_init(&bar[1], 1);
        tc::fence_mbar_init();
    }
    __syncthreads();
    auto fetch = [&](int tile, int buf) {  // one thread
        const int x = 2 * (CP::XOFF + (tile % ngroups) * C), img = tile / ngroups;
        mbar_expect(&bar[buf], (uint32_t)(CP::LAND * sizeof(float2)));
        for (int i = 0; i < CP::IN_ROWS / BR; ++i)
            tma_load3(fft_sh + CP::EX + buf * CP::LAND + i * BR * C, &tmap, x, CP::IN_Y0 + i * BR, img, &bar[buf]);
    };
    if (threadIdx.x == 0 && (int)blockIdx.x < ntiles) fetch(blockIdx.x, 0);
    bool ok = true;
    int it = 0;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++it) {
        const int buf = it & 1;
        // the other landing buffer was read in the previous iteration, before
        // at least one block barrier: it takes the next tile
        if (threadIdx.x == 0 && tile + (int)gridDim.x < ntiles) fetch(tile + gridDim.x, buf ^ 1);
        ok = tc::mbar_wait(&bar[buf], (uint32_t)((it >> 1) & 1), ok) && ok;
        float2 v[16];
        const float2 *in = fft_sh + CP::EX + buf * CP::LAND;
#pragma unroll
        for (int r = 0; r < 16; ++r) {
            if constexpr (DIR < 0)
                v[r] = (r >= 4 && r < 12) ? in[(t + N1 * r - n / 2) * C + c] : make_float2(0.f, 0.f);
            else
                v[r] = in[(t + N1 * r) * C + c];
        }
        if (threadIdx.x == 0) tma_store_wait_read();  // the previous output tile has left the exchange buffer
        __syncthreads();
        fft_core<N, DIR, L>(v, ex, c, t, tw);
        __syncthreads();
#pragma unroll
        for (int q = 0; q < 16 / L::R3; ++q)
#pragma unroll
            for (int j1 = 0; j1 < L::R3; ++j1) {
                const int Y = t + N1 * q + 256 * j1;
                if constexpr (DIR < 0) {
                    ex[Y * C + c] = v[q * L::R3 + j1];
                } else {
                    if (Y >= n / 2 && Y < n / 2 + n) ex[(Y - n / 2) * C + c] = v[q * L::R3 + j1];
                }
            }
        tc::fence_proxy_async();
        __syncthreads();
        if (threadIdx.x == 0) {
            const int x = 2 * (CP::XOFF + (tile % ngroups) * C), img = tile / ngroups;
            for (int i = 0; i < CP::OUT_ROWS / BR; ++i) tma_store3(&tmap, x, CP::OUT_Y0 + i * BR, img, ex + i * BR * C);
            asm volatile("cp.async.bulk.commit_group;\n" ::: "memory");
        }
    }
    if (threadIdx.x == 0) {
        asm volatile("cp.async.bulk.wait_group 0;\n" ::: "memory");  // the last tiles are written
        if (!ok) atomicAdd(err, 1);
    }
}

// ---------------------------------------------------------------------------
// Adjoint rows: rows Ya = n/2 + 2 pr and Ya + 1 of the column pass output
// (row pitch hp complex), Hermitian-extended to P points, one inverse FFT as
// A + i B; the centre outputs X in [n/2, 3n/2) are modulated, deapodised,
// scaled by c and added into rows 2 pr, 2 pr + 1 of u.
// ---------------------------------------------------------------------------
template <int N>
__global__ void __launch_bounds__(kRowThreads, 2)
    k_fft_rows_inv(const float2 *__restrict__ spec, float *__restrict__ u, const float *__restrict__ dp,
                   const float2 *__restrict__ tw, float cscale, int hp) {
    constexpr int N1 = N / 16, RP = kRowThreads / N1;
    using L = FftLayout<N, false, RP>;
    extern __shared__ float2 fft_sh[];
    const int n = N / 2;
    const int t = threadIdx.x % N1, c = threadIdx.x / N1;
    const int pr = blockIdx.x * RP + c;
    const long long img = blockIdx.y;
    const bool ok = pr < n / 2;
    const int ya = 2 * pr, yb = ya + 1, Ya = ya + n / 2;
    const float2 *ha = spec + img * N * hp + (long long)(ok ? Ya : n / 2) * hp;
    const float2 *hb = ha + hp;
    float2 v[16];
#pragma unroll
    for (int r = 0; r < 16; ++r) {
        const int k = t + N1 * r;
        float2 a, b;
        if (k <= n) {
            a = ha[k];
            b = hb[k];
            if (k == 0 || k == n) a.y = b.y = 0.f;
        } else {
            a = conj_(ha[N - k]);
            b = conj_(hb[N - k]);
        }
        v[r] = make_float2(a.x - b.y, a.y + b.x);  // A + i B
    }
    fft_core<N, 1, L>(v, fft_sh, c, t, tw);
    if (!ok) return;
    float *ua = u + (img * n + ya) * (long long)n;
    float *ub = ua + n;
    const float sa = ((Ya & 1) ? -dp[ya] : dp[ya]) * cscale;
    const float sb = ((Ya & 1) ? dp[yb] : -dp[yb]) * cscale;
#pragma unroll
    for (int q = 0; q < 16 / L::R3; ++q)
#pragma unroll
        for (int j1 = 0; j1 < L::R3; ++j1) {
            const int X = t + N1 * q + 256 * j1;
            const int x = X - n / 2;
            if (x >= 0 && x < n) {
                const float w = (X & 1) ? -__ldg(dp + x) : __ldg(dp + x);
                const float2 z = v[q * L::R3 + j1];
                ua[x] += z.x * w * sa;
                ub[x] += z.y * w * sb;
            }
        }
}

template <int N>
size_t rows_smem() {
    return sizeof(float2) * (size_t)FftLayout<N, false, kRowThreads / (N / 16)>::S * (kRowThreads / (N / 16));
}

// ---------------------------------------------------------------------------
// Residual rows of the inner step, fused: for two gathered rows a, b (rows of
// n complex values, already multiplied by (-1)^(k+1) shift(k) (pi/mu)/n):
//   x = Re IFFT_n(row)                                  (radonusfft.cu:98-102)
//   r(s) = x(s) (-1)^(s+1) / sqrt(n ntheta) - g(s)      (residual, admm.cu:92)
//   w(s) = (-1)^(s+1) r(s)                              (fftshift of adjR, radonusfft.cu:115)
//   R = FFT_n(w), k = 0 .. n/2                          (the adjoint's row transform)
// Re IFFT(a) + i Re IFFT(b) is the inverse FFT of Ha + i Hb (H = Hermitian
// part), and FFT(wa + i wb) splits into the two half spectra, so a row pair
// costs one inverse and one forward n-point FFT; the residual never goes to
// memory.  Rows are the flattened (slice, angle) index; N = n.
// ---------------------------------------------------------------------------
template <int N>
__global__ void __launch_bounds__(kRowThreads, 2)
    k_resid_rows(const float2 *__restrict__ rows, const float *__restrict__ gdata, float2 *__restrict__ out,
                 const float2 *__restrict__ tw, long long nrows, float scale) {
    constexpr int N1 = N / 16, RP = kRowThreads / N1;
    using L = FftLayout<N, false, RP>;
    extern __shared__ float2 fft_sh[];
    const int t = threadIdx.x % N1, c = threadIdx.x / N1;
    const long long ra = 2 * ((long long)blockIdx.x * RP + c), rb = ra + 1;
    const bool oka = ra < nrows, okb = rb < nrows;
    const float2 *ga = rows + (oka ? ra : 0) * N, *gb = rows + (okb ? rb : 0) * N;
    float2 v[16];
#pragma unroll
    for (int r = 0; r < 16; ++r) {  // Ha + i Hb at k = t + N1 r
        const int k = t + N1 * r, km = (N - k) & (N - 1);
        float2 a = make_float2(0.f, 0.f), b = make_float2(0.f, 0.f);
        if (oka) {
            const float2 p = ga[k], q = ga[km];
            a = make_float2(0.5f * (p.x + q.x), 0.5f * (p.y - q.y));
        }
        if (okb) {
            const float2 p = gb[k], q = gb[km];
            b = make_float2(0.5f * (p.x + q.x), 0.5f * (p.y - q.y));
        }
        v[r] = make_float2(a.x - b.y, a.y + b.x);
    }
    fft_core<N, 1, L>(v, fft_sh, c, t, tw);
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 16 / L::R3; ++q)
#pragma unroll
        for (int j1 = 0; j1 < L::R3; ++j1) fft_sh[c * L::S + t + N1 * q + 256 * j1] = v[q * L::R3 + j1];
    __syncthreads();
    const float *da = gdata + (oka ? ra : 0) * N, *db = gdata + (okb ? rb : 0) * N;
#pragma unroll
    for (int r = 0; r < 16; ++r) {
        const int sidx = t + N1 * r;
        const float2 x = fft_sh[c * L::S + sidx];
        const float sg = (sidx & 1) ? 1.f : -1.f;
        // as the separate passes: v = x (+-scale), r = v - g, w = (+-) r
        const float wa = oka ? sg * (sg * (x.x * scale) - da[sidx]) : 0.f;
        const float wb = okb ? sg * (sg * (x.y * scale) - db[sidx]) : 0.f;
        v[r] = make_float2(wa, wb);
    }
    __syncthreads();
    fft_core<N, -1, L>(v, fft_sh, c, t, tw);
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 16 / L::R3; ++q)
#pragma unroll
        for (int j1 = 0; j1 < L::R3; ++j1) fft_sh[c * L::S + t + N1 * q + 256 * j1] = v[q * L::R3 + j1];
    __syncthreads();
    constexpr int HN = N / 2 + 1;
    for (int k = t; k < HN; k += N1) {
        const float2 zk = fft_sh[c * L::S + k], zm = fft_sh[c * L::S + ((N - k) & (N - 1))];
        if (oka) out[ra * HN + k] = make_float2(0.5f * (zk.x + zm.x), 0.5f * (zk.y - zm.y));
        if (okb) out[rb * HN + k] = make_float2(0.5f * (zk.y + zm.y), 0.5f * (zm.x - zk.x));
    }
}

template <int N>
void resid_n(const float2 *rows, const float *gdata, float2 *out, const float2 *tw, long long nrows, float scale,
             cudaStream_t s) {
    constexpr int N1 = N / 16, RP = kRowThreads / N1;
    const long long npairs = (nrows + 1) / 2;
    const long long nblk = (npairs + RP - 1) / RP;
    if (nblk > 2147483647LL) throw Error(1, "residual rows: too many rows");
    k_resid_rows<N><<<(unsigned)nblk, kRowThreads, rows_smem<N>(), s>>>(rows, gdata, out, tw, nrows, scale);
    LAUNCH_CHECK("k_resid_rows");
}

template <int N>
void set_attrs_n() {
    CUDA_CHECK(cudaFuncSetAttribute(k_resid_rows<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rows_smem<N>()));
    CUDA_CHECK(cudaFuncSetAttribute(k_fft_rows_fwd<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rows_smem<N>()));
    CUDA_CHECK(cudaFuncSetAttribute(k_fft_rows_inv<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rows_smem<N>()));
    CUDA_CHECK(cudaFuncSetAttribute(k_fft_cols<N, kColC, -1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)ColPass<N, kColC, -1>::SMEM));
    CUDA_CHECK(cudaFuncSetAttribute(k_fft_cols<N, kColC, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)ColPass<N, kColC, 1>::SMEM));
}

int sm_count() {
    static int nsm = 0;
    if (nsm == 0) {
        int dev = 0;
        CUDA_CHECK(cudaGetDevice(&dev));
        CUDA_CHECK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    }
    return nsm;
}

template <int N, int DIR>
void launch_cols(const CUtensorMap &map, const float2 *tw, int nimg, int *err, cudaStream_t s) {
    const int ngroups = (N / 2 + 1 + kColC - 1) / kColC;
    const long long ntiles = (long long)ngroups * nimg;
    if (ntiles > 2147483647LL) throw Error(1, "pad FFT: too many column tiles");
    const int grid = (int)std::min<long long>(ntiles, sm_count());
    k_fft_cols<N, kColC, DIR><<<grid, kColC * (N / 16), ColPass<N, kColC, DIR>::SMEM, s>>>(map, tw, ngroups,
                                                                                         (int)ntiles, err);
    LAUNCH_CHECK(DIR < 0 ? "k_fft_cols (forward)" : "k_fft_cols (inverse)");
}

template <int N>
void fwd_n(const float *u, float2 *spec, int nimg, const float *deapod, const float2 *tw, const CUtensorMap &map,
           int *err, const UsGeo &g, cudaStream_t s) {
    constexpr int N1 = N / 16, RP = kRowThreads / N1;
    const int n = N / 2;
    const float inv4n2 = (float)(1.0 / (4.0 * n * (double)n));
    dim3 gr((n / 2 + RP - 1) / RP, nimg);
    k_fft_rows_fwd<N><<<gr, kRowThreads, rows_smem<N>(), s>>>(u, spec, deapod, tw, g, inv4n2);
    LAUNCH_CHECK("k_fft_rows_fwd");
    launch_cols<N, -1>(map, tw, nimg, err, s);
}

template <int N>
void inv_n(float2 *spec, float *u, int nimg, float cscale, const float *deapod, const float2 *tw,
           const CUtensorMap &map, int *err, int hpitch, cudaStream_t s) {
    constexpr int N1 = N / 16, RP = kRowThreads / N1;
    const int n = N / 2;
    launch_cols<N, 1>(map, tw, nimg, err, s);
    dim3 gr((n / 2 + RP - 1) / RP, nimg);
    k_fft_rows_inv<N><<<gr, kRowThreads, rows_smem<N>(), s>>>(spec, u, deapod, tw, cscale, hpitch);
    LAUNCH_CHECK("k_fft_rows_inv");
}

PFN_cuTensorMapEncodeTiled_v12000 tmap_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    if (!encode) {
        cudaDriverEntryPointQueryResult q;
        CUDA_CHECK(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", (void **)&encode, 12000,
                                                    cudaEnableDefault, &q));
        if (q != cudaDriverEntryPointSuccess || !encode) throw Error(1, "cuTensorMapEncodeTiled unavailable");
    }
    return encode;
}

// float view [nimg][rows][row_floats] (pitches in bytes), boxes of 8 floats x
// min(n, 256) rows x 1 image
void encode_cols_map(CUtensorMap *map, void *base, long long row_floats, long long rows, long long nimg,
                     long long row_pitch, long long img_pitch, int n, const char *what) {
    const cuuint64_t dims[3] = {(cuuint64_t)row_floats, (cuuint64_t)rows, (cuuint64_t)nimg};
    const cuuint64_t strides[2] = {(cuuint64_t)row_pitch, (cuuint64_t)img_pitch};
    const cuuint32_t box[3] = {2 * kColC, (cuuint32_t)(n < 256 ? n : 256), 1};
    const cuuint32_t es[3] = {1, 1, 1};
    const CUresult r = tmap_encoder()(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, base, dims, strides, box, es,
                                      CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                      CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) throw Error(1, std::string("cuTensorMapEncodeTiled failed for ") + what);
}

}  // namespace

// P <= 2048: the column passes' two landing tiles and exchange buffer fit in
// shared memory up to that size
bool pad_fft_supported(int P) { return P >= 256 && P <= 2048 && (P & (P - 1)) == 0; }

void pad_fft_prepare() {
    set_attrs_n<256>();
    set_attrs_n<512>();
    set_attrs_n<1024>();
    set_attrs_n<2048>();
}

std::vector<float2> pad_fft_twiddles(int P) {
    const int N1 = P / 16, R3 = P / 256;
    std::vector<float2> w((size_t)P + 16 * R3);
    const double pi = 3.14159265358979323846;
    auto cis = [&](long long e) {
        const double a = -2.0 * pi * (double)(e % P) / (double)P;
        return make_float2((float)std::cos(a), (float)std::sin(a));
    };
    for (int k2 = 0; k2 < 16; ++k2)
        for (int t = 0; t < N1; ++t) w[(size_t)k2 * N1 + t] = cis((long long)t * k2);
    for (int j2 = 0; j2 < 16; ++j2)
        for (int m1 = 0; m1 < R3; ++m1) w[(size_t)P + j2 * R3 + m1] = cis(16LL * m1 * j2);
    return w;
}

void make_pad_fft_maps(CUtensorMap *fwd, CUtensorMap *inv, float2 *spec, int nimg, const UsGeo &g) {
    // forward: the halo-padded window [P + 2 kHalo rows][2 qp floats]
    encode_cols_map(fwd, spec, 2LL * g.qp, g.P + 2LL * kHalo, nimg, 8LL * g.qp, 8LL * g.img_fwd, g.n,
                    "the forward column FFT");
    // inverse: Hermitian half planes [P rows][2 hpitch floats]
    encode_cols_map(inv, spec, 2LL * g.hpitch, g.P, nimg, 8LL * g.hpitch, 8LL * g.P * g.hpitch, g.n,
                    "the inverse column FFT");
}

void launch_pad_fft_fwd(const float *u, float2 *spec, int nimg, const float *deapod, const float2 *tw,
                        const CUtensorMap &map, int *err, const UsGeo &g, cudaStream_t s) {
    if (nimg > 65535) throw Error(1, "pad FFT: too many images per batch");
    switch (g.P) {
        case 256: fwd_n<256>(u, spec, nimg, deapod, tw, map, err, g, s); break;
        case 512: fwd_n<512>(u, spec, nimg, deapod, tw, map, err, g, s); break;
        case 1024: fwd_n<1024>(u, spec, nimg, deapod, tw, map, err, g, s); break;
        case 2048: fwd_n<2048>(u, spec, nimg, deapod, tw, map, err, g, s); break;
        default: throw Error(1, "pad FFT: unsupported grid size");
    }
}

bool resid_rows_supported(int n) { return n >= 256 && n <= 1024 && (n & (n - 1)) == 0; }

// tw_n: the twiddle table of the n-point transforms, pad_fft_twiddles(n)
void launch_resid_rows(const float2 *rows, const float *gdata, float2 *out, const float2 *tw_n, int zb,
                       const UsGeo &g, cudaStream_t s) {
    const long long nrows = (long long)zb * g.ntheta;
    const float scale = (float)(1.0 / std::sqrt((double)g.n * (double)g.ntheta));
    switch (g.n) {
        case 256: resid_n<256>(rows, gdata, out, tw_n, nrows, scale, s); break;
        case 512: resid_n<512>(rows, gdata, out, tw_n, nrows, scale, s); break;
        case 1024: resid_n<1024>(rows, gdata, out, tw_n, nrows, scale, s); break;
        default: throw Error(1, "residual rows: unsupported detector width");
    }
}

void launch_pad_fft_inv_accum(float2 *spec, float *u, int zb, float tau, const float *deapod, const float2 *tw,
                              const CUtensorMap &map, int *err, const UsGeo &g, cudaStream_t s) {
    const int nimg = zb * g.m;
    if (nimg > 65535) throw Error(1, "pad FFT: too many images per batch");
    // the scale of the C2R path's crop (1/sqrt(n ntheta) / (4 n^2)) times tau
    const double scale = 1.0 / std::sqrt((double)g.n * (double)g.ntheta);
    const float c = (float)(tau * scale / (4.0 * g.n * (double)g.n));
    switch (g.P) {
        case 256: inv_n<256>(spec, u, nimg, c, deapod, tw, map, err, g.hpitch, s); break;
        case 512: inv_n<512>(spec, u, nimg, c, deapod, tw, map, err, g.hpitch, s); break;
        case 1024: inv_n<1024>(spec, u, nimg, c, deapod, tw, map, err, g.hpitch, s); break;
        case 2048: inv_n<2048>(spec, u, nimg, c, deapod, tw, map, err, g.hpitch, s); break;
        default: throw Error(1, "pad FFT: unsupported grid size");
    }
}

}  // namespace rectv
