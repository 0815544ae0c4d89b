// USFFT Radon transform kernels for the temporal-basis operator R_apr and its
// adjoint, specialised for sm_103a.
//
// The reference (radonusfft.cu:77-135, operators.cu:6-58) runs, for every
// basis function i, a full USFFT (2D FFT of a complex image, 81-tap gather
// from global memory, 1D FFT) and mixes time samples and bases around it.
// Everything between the FFTs is linear, so the same result is computed here
// with one real-input 2D FFT per time sample, one gather/scatter pass over
// all time samples at once, and one row FFT per (slice, angle):
//
//   R_apr u (theta, s) = Re IFFT_k[ (-1)^(k+1) shiftfwd(k)
//                           sum_j K'(theta, j) Gather_theta,k( FFT2(pad(u_j)) ) ]
//   K'(theta, j) = ntheta/sqrt(m) sum_i phi_i(theta) conj(phi_i(t_j))
//
// and the adjoint scatters conj(K'(theta, j)) E(theta, k) into time sample j's
// grid.  The gather reads a shared-memory tile holding all time samples of a
// (T+8)^2 patch of the oversampled spectrum; one warp lane per (time sample,
// re/im) makes every tap a conflict-free 128-byte shared-memory row read.
#include <cuda_runtime.h>

#include "rectv_internal.cuh"

namespace rectv {

namespace {

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// Position of polar sample (theta, k): identical float operation sequence to
// the host plan (plan.cpp) and to takexy (kernels_radonusfft.cuh:73-78).
__device__ __forceinline__ void sample_pos(int k, float2 sc, const UsGeo &g, float &x0, float &y0,
                                           int &fx, int &fy) {
    const float q = __fdiv_rn((float)(k - g.n / 2), (float)g.n);
    x0 = __fmul_rn(q, sc.x);
    y0 = __fmul_rn(q, sc.y);
    if (x0 >= 0.5f) x0 = 0.5f - 1e-5f;
    if (y0 >= 0.5f) y0 = 0.5f - 1e-5f;
    fx = (int)floorf(__fmul_rn(g.tn, x0));
    fy = (int)floorf(__fmul_rn(g.tn, y0));
}

// Separable Gaussian weights exp(-pi^2/mu d^2) of the 9 taps per axis
// (gather, kernels_radonusfft.cuh:116-118; pi/mu and 1/n are applied once).
__device__ __forceinline__ void tap_weights(int f, float p0, const UsGeo &g, float (&e)[kTaps]) {
#pragma unroll
    for (int i = 0; i < kTaps; ++i) {
        const float d = (float)(f - kR + i) * g.inv2n - p0;
        e[i] = __expf(-g.wexp * d * d);
    }
}

}  // namespace

// ---------------------------------------------------------------------------
// Forward: deapodise, zero-pad to P x P and modulate by (-1)^(X+Y)
// (divphi + fftshift, kernels_radonusfft.cuh:4-38), writing the in-place R2C
// layout (rows of P+2 floats).
// ---------------------------------------------------------------------------
__global__ void k_deapod_pad(const float *__restrict__ u, float *__restrict__ spec,
                             const float *__restrict__ dp, int n, int P, float inv4n2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;  // float pair in the row
    const int Y = blockIdx.y;
    const long long img = blockIdx.z;
    const int npair = (P + 2) / 2;
    if (i >= npair) return;
    const int X = 2 * i;
    float2 v = make_float2(0.f, 0.f);
    const int y = Y - n / 2;
    if (y >= 0 && y < n) {
        const float *row = u + (img * n + y) * (long long)n;
        const float sy = (Y & 1) ? -dp[y] * inv4n2 : dp[y] * inv4n2;
        const int x0 = X - n / 2, x1 = x0 + 1;
        if (x0 >= 0 && x0 < n) v.x = row[x0] * dp[x0] * sy;   // X even: +1
        if (x1 >= 0 && x1 < n) v.y = -row[x1] * dp[x1] * sy;  // X+1 odd: -1
    }
    reinterpret_cast<float2 *>(spec + img * (long long)P * (P + 2) + (long long)Y * (P + 2))[i] = v;
}

void launch_deapod_pad(const float *u, float *spec, int nimg, const float *deapod, const UsGeo &g,
                       cudaStream_t s) {
    const int npair = (g.P + 2) / 2;
    dim3 bs(256), gs((npair + 255) / 256, g.P, nimg);
    const float inv4n2 = (float)(1.0 / (4.0 * g.n * (double)g.n));
    k_deapod_pad<<<gs, bs, 0, s>>>(u, spec, deapod, g.n, g.P, inv4n2);
    LAUNCH_CHECK("k_deapod_pad");
}

// ---------------------------------------------------------------------------
// Forward gather (gather TOMO_FWD, kernels_radonusfft.cuh:81-144, fused with
// the basis sum of operators.cu:143-152 and shift/fftshift of
// radonusfft.cu:96-97).  One block per (work item, slice); a work item is a
// tile of the spectrum and up to `cap` samples whose stencil centre lies in
// it.  jbase selects a group of MP time samples (m > 16 runs several passes,
// accumulating into rows).
// ---------------------------------------------------------------------------
template <int MP, int T>
__global__ void __launch_bounds__(256)
    k_gather_fwd(const float2 *__restrict__ spec, float2 *__restrict__ rows,
                 const uint32_t *__restrict__ pts, const int4 *__restrict__ items,
                 const float2 *__restrict__ sincos, const float2 *__restrict__ kmat,
                 const float2 *__restrict__ shiftf, UsGeo g, int jbase, int accumulate,
                 int *__restrict__ err) {
    constexpr int TW = T + 2 * kR;
    constexpr int LPP = 2 * MP;
    constexpr int GPW = 32 / LPP;
    extern __shared__ float2 sm[];  // [NC][MP]
    const int4 it = items[blockIdx.x];
    const int z = blockIdx.y;
    const int tyi = it.x / g.NT, txi = it.x - tyi * g.NT;
    const int P = g.P, half = P / 2;
    const float2 *img0 = spec + (long long)z * g.m * g.img_fwd;

    // ---- stage the tile: unit = (row, quad of 4 cells, time sample) ----
    {
        constexpr int NQ = TW / 4;
        const int nunits = TW * NQ * MP;
        for (int u = threadIdx.x; u < nunits; u += blockDim.x) {
            const int j = u % MP;
            const int rq = u / MP;
            const int row = rq / NQ, q = rq - row * NQ;
            const int jg = jbase + j;
            int KY = tyi * T - kR + row;
            KY += (KY < 0) ? P : 0;
            KY -= (KY >= P) ? P : 0;
            float2 v[4];
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                float2 w = make_float2(0.f, 0.f);
                if (jg < g.m) {
                    int KX = txi * T - kR + 4 * q + c;
                    KX += (KX < 0) ? P : 0;
                    KX -= (KX >= P) ? P : 0;
                    const float2 *im = img0 + (long long)jg * g.img_fwd;
                    if (KX <= half) {
                        w = __ldg(im + (long long)KY * g.hp + KX);
                    } else {  // Hermitian symmetry of the real-input FFT
                        const int KYm = KY ? P - KY : 0;
                        w = __ldg(im + (long long)KYm * g.hp + (P - KX));
                        w.y = -w.y;
                    }
                    if ((KX + KY) & 1) {  // post-FFT fftshift (-1)^(X+Y)
                        w.x = -w.x;
                        w.y = -w.y;
                    }
                }
                v[c] = w;
            }
#pragma unroll
            for (int c = 0; c < 4; ++c) sm[(row * TW + 4 * q + c) * MP + j] = v[c];
        }
    }
    __syncthreads();

    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int grp = lane / LPP, l = lane - grp * LPP, j = l >> 1;
    const int jg = jbase + j;
    const float *smf = reinterpret_cast<const float *>(sm);
    const int count = it.z;
    const unsigned full = 0xffffffffu;
    for (int p0 = wid * GPW; p0 < count; p0 += nw * GPW) {
        const int p = p0 + grp;
        bool valid = p < count;
        const uint32_t id = __ldg(pts + it.y + (valid ? p : p0));
        const int th = id / (uint32_t)g.n;
        const int k = id - th * g.n;
        float x0, y0;
        int fx, fy;
        sample_pos(k, __ldg(sincos + th), g, x0, y0, fx, fy);
        const int lx0 = g.n + fx - txi * T;
        const int ly0 = g.n + fy - tyi * T;
        if (lx0 < 0 || lx0 >= T || ly0 < 0 || ly0 >= T) {  // host/device bin disagreement
            if (valid && l == 0) atomicAdd(err, 1);
            valid = false;
        }
        float ex[kTaps], ey[kTaps];
        tap_weights(fx, x0, g, ex);
        tap_weights(fy, y0, g, ey);
        const int cbase = valid ? (ly0 * TW + lx0) : 0;
        const float *b0 = smf + cbase * LPP + l;
        float acc = 0.f;
#pragma unroll
        for (int a = 0; a < kTaps; ++a) {
            float ra = 0.f;
#pragma unroll
            for (int b = 0; b < kTaps; ++b) ra = fmaf(ex[b], b0[(a * TW + b) * LPP], ra);
            acc = fmaf(ey[a], ra, acc);
        }
        // time-sample mixing: sum_j K'(theta, j) H_j  (re/im live in lane pairs)
        const float2 kv = (jg < g.m) ? __ldg(kmat + (long long)th * g.m + jg) : make_float2(0.f, 0.f);
        const float part = __shfl_xor_sync(full, acc, 1);
        float val = (l & 1) ? (kv.x * acc + kv.y * part) : (kv.x * acc - kv.y * part);
#pragma unroll
        for (int o = 2; o < LPP; o <<= 1) val += __shfl_xor_sync(full, val, o);
        const float oth = __shfl_xor_sync(full, val, 1);
        if (valid && l == 0) {
            float2 sh = __ldg(shiftf + k);
            const float c = (k & 1) ? g.cw : -g.cw;  // (-1)^(k+1) and (pi/mu)/n
            sh.x *= c;
            sh.y *= c;
            float2 r = cmul(make_float2(val, oth), sh);
            float2 *dst = rows + ((long long)z * g.ntheta + th) * g.n + k;
            if (accumulate) {
                const float2 o = *dst;
                r.x += o.x;
                r.y += o.y;
            }
            *dst = r;
        }
    }
}

static int mp_for(int m) {
    int mp = 1;
    while (mp < m && mp < 16) mp <<= 1;
    return mp;
}

size_t gather_fwd_smem(const UsGeo &g) {
    return (size_t)(g.T + 2 * kR) * (g.T + 2 * kR) * mp_for(g.m) * sizeof(float2);
}
size_t scatter_adj_smem(const UsGeo &g) { return (size_t)g.T * g.T * mp_for(g.m) * sizeof(float2); }

template <int MP, int T>
static void gather_fwd_t(const float2 *spec, float2 *rows, int zb, const GeoDev &gd, const UsGeo &g,
                         int jbase, int accumulate, int *err, cudaStream_t s) {
    const size_t smem = (size_t)(T + 2 * kR) * (T + 2 * kR) * MP * sizeof(float2);
    dim3 gs(gd.n_fwd_items, zb);
    k_gather_fwd<MP, T><<<gs, 256, smem, s>>>(spec, rows, gd.fwd_pts, gd.fwd_items, gd.sincos, gd.kmat,
                                              gd.shiftfwd, g, jbase, accumulate, err);
    LAUNCH_CHECK("k_gather_fwd");
}

// rows[z][theta][0] = 0: the k = 0 sample is zeroed by the reference
// (kernels_radonusfft.cuh:138-142) and has no entry in the plan.
__global__ void k_zero_k0(float2 *rows, long long nrows, int n) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < nrows) rows[i * n] = make_float2(0.f, 0.f);
}

void launch_gather_fwd(const float2 *spec, float2 *rows, int zb, const GeoDev &gd, const UsGeo &g,
                       cudaStream_t s) {
    const long long nrows = (long long)zb * g.ntheta;
    k_zero_k0<<<(unsigned)((nrows + 255) / 256), 256, 0, s>>>(rows, nrows, g.n);
    LAUNCH_CHECK("k_zero_k0");
    if (g.T != 16) throw Error(1, "tile size must be 16");
    const int mp = mp_for(g.m);
    for (int jb = 0; jb < g.m; jb += 16) {
        const int acc = jb > 0;
        switch (mp) {
            case 1: gather_fwd_t<1, 16>(spec, rows, zb, gd, g, jb, acc, gd.err, s); break;
            case 2: gather_fwd_t<2, 16>(spec, rows, zb, gd, g, jb, acc, gd.err, s); break;
            case 4: gather_fwd_t<4, 16>(spec, rows, zb, gd, g, jb, acc, gd.err, s); break;
            case 8: gather_fwd_t<8, 16>(spec, rows, zb, gd, g, jb, acc, gd.err, s); break;
            default: gather_fwd_t<16, 16>(spec, rows, zb, gd, g, jb, acc, gd.err, s); break;
        }
    }
}

// ---------------------------------------------------------------------------
// Forward epilogue after the inverse row FFT: fftshift (-1)^(s+1), 1/sqrt(n
// ntheta) (radonusfft.cu:100-102), real part (addreal, kernels_operators.cuh:75-84).
// residual != 0: out = R u - gdata (lin, admm.cu:92); else out = tau R u.
// ---------------------------------------------------------------------------
__global__ void k_finish_fwd(const float2 *__restrict__ rows, const float *__restrict__ gdata,
                             float *__restrict__ out, long long total, int n, float scale, float tau,
                             int residual) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= total) return;
    const int sidx = (int)(i % n);
    const float v = rows[i].x * ((sidx & 1) ? scale : -scale);
    if (residual) {
        out[i] = v - gdata[i];
    } else {
        out[i] = tau * v;
    }
}

void launch_finish_fwd(const float2 *rows, const float *gdata, float *out, int zb, float tau,
                       int residual, const UsGeo &g, cudaStream_t s) {
    const long long total = (long long)zb * g.ntheta * g.n;
    const float scale = (float)(1.0 / std::sqrt((double)g.n * (double)g.ntheta));
    k_finish_fwd<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(rows, gdata, out, total, g.n, scale, tau,
                                                                 residual);
    LAUNCH_CHECK("k_finish_fwd");
}

// ---------------------------------------------------------------------------
// Adjoint prologue: fftshift (-1)^(s+1) of the real residual rows into the
// in-place R2C layout (rows of 2(n/2+1) floats) (radonusfft.cu:115).
// ---------------------------------------------------------------------------
__global__ void k_adj_prep(const float *__restrict__ h, float *__restrict__ rowsr, long long nrows,
                           int n) {
    const int rs = 2 * (n / 2 + 1);
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long total = nrows * rs;
    if (i >= total) return;
    const long long r = i / rs;
    const int sidx = (int)(i - r * rs);
    float v = 0.f;
    if (sidx < n) {
        v = h[r * n + sidx];
        v = (sidx & 1) ? v : -v;
    }
    rowsr[i] = v;
}

void launch_adj_prep(const float *h, float *rowsr, int zb, const UsGeo &g, cudaStream_t s) {
    const long long nrows = (long long)zb * g.ntheta;
    const long long total = nrows * (2 * (g.n / 2 + 1));
    k_adj_prep<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(h, rowsr, nrows, g.n);
    LAUNCH_CHECK("k_adj_prep");
}

// Zero the core cells of tiles that several scatter blocks accumulate into.
__global__ void k_zero_split(float2 *spec, const int *__restrict__ tiles, int T, int NT, int P,
                             long long img_adj) {
    const int t = tiles[blockIdx.x];
    const long long img = blockIdx.y;
    const int tyi = t / NT, txi = t - tyi * NT;
    for (int c = threadIdx.x; c < T * T; c += blockDim.x) {
        const int ly = c / T, lx = c - ly * T;
        const int KY = tyi * T + ly, KX = txi * T + lx;
        if (KY < P && KX < P) spec[img * img_adj + (long long)KY * P + KX] = make_float2(0.f, 0.f);
    }
}

void launch_zero_split(float2 *spec, int zb, const GeoDev &gd, const UsGeo &g, cudaStream_t s) {
    if (gd.n_split_tiles == 0) return;
    dim3 gs(gd.n_split_tiles, zb * g.m);
    k_zero_split<<<gs, 256, 0, s>>>(spec, gd.split_tiles, g.T, g.NT, g.P, g.img_adj);
    LAUNCH_CHECK("k_zero_split");
}

// ---------------------------------------------------------------------------
// Adjoint scatter (gather TOMO_ADJ + wrap TOMO_ADJ, kernels_radonusfft.cuh:
// 40-64,81-144, fused with shift/fftshift of radonusfft.cu:115-121, the basis
// weights of operators.cu:171-176 and the pre-IFFT fftshift).  One block per
// (work item, slice) owns a T x T tile of the periodic P x P grid and
// accumulates every sample whose stencil touches it in shared memory, then
// stores the tile once (or adds it, for tiles split over several blocks).
// ---------------------------------------------------------------------------
template <int MP, int T>
__global__ void __launch_bounds__(256)
    k_scatter_adj(const float2 *__restrict__ rowsc, float2 *__restrict__ spec,
                  const uint32_t *__restrict__ pts, const int4 *__restrict__ items,
                  const float2 *__restrict__ sincos, const float2 *__restrict__ kmat,
                  const float2 *__restrict__ shifta, UsGeo g, int jbase) {
    constexpr int LPP = 2 * MP;
    constexpr int GPW = 32 / LPP;
    extern __shared__ float2 acc[];  // [T*T][MP]
    float *accf = reinterpret_cast<float *>(acc);
    for (int i = threadIdx.x; i < T * T * LPP; i += blockDim.x) accf[i] = 0.f;
    __syncthreads();
    const int4 it = items[blockIdx.x];
    const int z = blockIdx.y;
    const int tyi = it.x / g.NT, txi = it.x - tyi * g.NT;
    const int P = g.P, half = P / 2, hn = g.n / 2 + 1;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int grp = lane / LPP, l = lane - grp * LPP, j = l >> 1, comp = l & 1;
    const int jg = jbase + j;
    const int count = it.z;
    const float2 *rz = rowsc + (long long)z * g.ntheta * hn;
    for (int p0 = wid * GPW; p0 < count; p0 += nw * GPW) {
        const int p = p0 + grp;
        const bool valid = p < count;
        const uint32_t id = __ldg(pts + it.y + (valid ? p : p0));
        const int th = id / (uint32_t)g.n;
        const int k = id - th * g.n;
        float x0, y0;
        int fx, fy;
        sample_pos(k, __ldg(sincos + th), g, x0, y0, fx, fy);
        int dx = g.n + fx - kR - txi * T;
        int dy = g.n + fy - kR - tyi * T;
        dx += (dx < -half) ? P : 0;
        dx -= (dx > half) ? P : 0;
        dy += (dy < -half) ? P : 0;
        dy -= (dy > half) ? P : 0;
        // E = (-1)^(k+1) shiftadj(k) FFT(row)(k) (pi/mu)/n  (Hermitian row spectrum)
        float2 R = (k <= g.n / 2) ? __ldg(rz + (long long)th * hn + k)
                                  : __ldg(rz + (long long)th * hn + (g.n - k));
        if (k > g.n / 2) R.y = -R.y;
        const float2 S = __ldg(shifta + k);
        float2 E = cmul(R, S);
        const float c = (k & 1) ? g.cw : -g.cw;
        E.x *= c;
        E.y *= c;
        const float2 kv = (jg < g.m) ? __ldg(kmat + (long long)th * g.m + jg) : make_float2(0.f, 0.f);
        float qv = comp ? (kv.x * E.y - kv.y * E.x) : (kv.x * E.x + kv.y * E.y);  // conj(K') E
        if (!valid) qv = 0.f;
        float ex[kTaps], ey[kTaps];
        tap_weights(fx, x0, g, ex);
        tap_weights(fy, y0, g, ey);
#pragma unroll
        for (int a = 0; a < kTaps; ++a) {
            const int ly = dy + a;
            if ((unsigned)ly < (unsigned)T) {
                const float wa = ey[a] * qv;
#pragma unroll
                for (int b = 0; b < kTaps; ++b) {
                    const int lx = dx + b;
                    if ((unsigned)lx < (unsigned)T) atomicAdd(&accf[(ly * T + lx) * LPP + l], ex[b] * wa);
                }
            }
        }
    }
    __syncthreads();
    // ---- flush: unit = (row, quad, time sample); pre-IFFT fftshift sign ----
    constexpr int NQ = T / 4;
    const int nunits = T * NQ * MP;
    const int split = it.w;
    for (int u = threadIdx.x; u < nunits; u += blockDim.x) {
        const int jj = u % MP;
        const int rq = u / MP;
        const int row = rq / NQ, q = rq - row * NQ;
        const int jgg = jbase + jj;
        if (jgg >= g.m) continue;
        const int KY = tyi * T + row;
        if (KY >= P) continue;  // partial last tile row
        float2 *dst = spec + ((long long)z * g.m + jgg) * g.img_adj + (long long)KY * P + txi * T + 4 * q;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const int KX = txi * T + 4 * q + c;
            if (KX >= P) break;
            float2 v = acc[(row * T + 4 * q + c) * MP + jj];
            if ((KX + KY) & 1) {
                v.x = -v.x;
                v.y = -v.y;
            }
            if (split) {
                atomicAdd(&dst[c].x, v.x);
                atomicAdd(&dst[c].y, v.y);
            } else {
                dst[c] = v;
            }
        }
    }
}

template <int MP, int T>
static void scatter_adj_t(const float2 *rowsc, float2 *spec, int zb, const GeoDev &gd,
                          const UsGeo &g, int jbase, cudaStream_t s) {
    const size_t smem = (size_t)T * T * MP * sizeof(float2);
    dim3 gs(gd.n_adj_items, zb);
    k_scatter_adj<MP, T><<<gs, 256, smem, s>>>(rowsc, spec, gd.adj_pts, gd.adj_items, gd.sincos, gd.kmat,
                                               gd.shiftadj, g, jbase);
    LAUNCH_CHECK("k_scatter_adj");
}

void launch_scatter_adj(const float2 *rowsc, float2 *spec, int zb, const GeoDev &gd,
                        const UsGeo &g, cudaStream_t s) {
    if (g.T != 16) throw Error(1, "tile size must be 16");
    const int mp = mp_for(g.m);
    for (int jb = 0; jb < g.m; jb += 16) {
        switch (mp) {
            case 1: scatter_adj_t<1, 16>(rowsc, spec, zb, gd, g, jb, s); break;
            case 2: scatter_adj_t<2, 16>(rowsc, spec, zb, gd, g, jb, s); break;
            case 4: scatter_adj_t<4, 16>(rowsc, spec, zb, gd, g, jb, s); break;
            case 8: scatter_adj_t<8, 16>(rowsc, spec, zb, gd, g, jb, s); break;
            default: scatter_adj_t<16, 16>(rowsc, spec, zb, gd, g, jb, s); break;
        }
    }
}

// ---------------------------------------------------------------------------
// Adjoint epilogue after the inverse 2D FFT: post-FFT fftshift, crop and
// deapodisation (divphi TOMO_ADJ), 1/sqrt(n ntheta) (radonusfft.cu:129-132),
// real part accumulated with tau (addreal, operators.cu:178).
// ---------------------------------------------------------------------------
__global__ void k_crop_accum(const float2 *__restrict__ spec, float *__restrict__ u,
                             const float *__restrict__ dp, int n, int P, long long img_adj, float c) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    const long long img = blockIdx.z;
    if (x >= n) return;
    const int X = x + n / 2, Y = y + n / 2;
    float v = spec[img * img_adj + (long long)Y * P + X].x;
    v = ((X + Y) & 1) ? -v : v;
    u[(img * n + y) * n + x] += c * v * dp[x] * dp[y];
}

void launch_crop_accum(const float2 *spec, float *u, int zb, float tau, const float *deapod,
                       const UsGeo &g, cudaStream_t s) {
    dim3 gs((g.n + 255) / 256, g.n, zb * g.m);
    const double scale = 1.0 / std::sqrt((double)g.n * (double)g.ntheta);
    const float c = (float)(tau * scale / (4.0 * g.n * (double)g.n));
    k_crop_accum<<<gs, 256, 0, s>>>(spec, u, deapod, g.n, g.P, g.img_adj, c);
    LAUNCH_CHECK("k_crop_accum");
}

template <int MP, int T>
static void set_attrs() {
    const int fs = (int)((T + 2 * kR) * (T + 2 * kR) * MP * sizeof(float2));
    const int as = (int)(T * T * MP * sizeof(float2));
    CUDA_CHECK(cudaFuncSetAttribute(k_gather_fwd<MP, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, fs));
    CUDA_CHECK(cudaFuncSetAttribute(k_scatter_adj<MP, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, as));
}

void usfft_prepare() {
    set_attrs<1, 16>();
    set_attrs<2, 16>();
    set_attrs<4, 16>();
    set_attrs<8, 16>();
    set_attrs<16, 16>();
}

}  // namespace rectv
