// USFFT gather and scatter for scans that revisit their directions.
//
// A scan over several half-turns sees every direction (theta modulo pi) more
// than once: rays theta, theta + pi, theta + 2 pi, ... sample the same points
// of the frequency plane (sample k of ray theta + pi is sample n - k of ray
// theta), and only their time weights K'(theta, j) differ.  The Gaussian
// interpolation (gather, kernels_radonusfft.cuh:81-144: 81 taps per sample)
// is linear and does not depend on a ray's time, so it is done once per
// position p = (direction d, 1 <= q < n) and time sample j, and the rays of
// the position are formed from it (the basis sums of operators.cu:143-152
// and 171-176 as the mixing K'):
//
//   forward:  S_j(p) = sum_taps w(p, c) F_j(c)
//             row(theta, k) = f(k) sum_j K'(theta, j) S_j(p)        (every ray theta of p)
//   adjoint:  E_j(p) = sum_{rays theta of p} conj K'(theta, j) f'(k) e(theta, k)
//             F_j(c) += sum_p w(p, c) E_j(p)
//
// with k = q for the rays of the representative's orientation and k = n - q
// for the opposite ones, f(k) = (-1)^(k+1) shiftfwd(k) (pi/mu)/n and f'(k) the
// same with shiftadj.
//
// The rays of a direction are grouped when their angles agree to the float32
// resolution of the input angles (2e-3 grid cells at the spectrum's edge);
// ray theta's own samples then lie delta = (q - n/2)/n tau_theta cells
// across the direction from the shared positions (DirPlan::tau).  Both
// kernels take that offset to first order: the forward interpolates S and
// its derivative across the direction, S_perp = sum_taps dw/dperp F, and ray
// theta reads S + delta S_perp; the adjoint scatters E and E_perp =
// sum_theta delta conj K' f' e with the weights w and dw/dperp.  The error
// left is O(delta^2) (the zeroth-order grouping alone errs by ~2e-4 relative
// at n = 1024 on white-noise spectra).
//
// At 2880 angles over 8 half-turns there are 360 directions: one eighth of
// the taps of the per-ray kernels, and the [ntheta x M] basis contraction
// becomes an 8-ray x 16-time-sample mix per position (FP32 on the CUDA
// cores: 16 complex products per ray sample, against 1296 for the taps of the
// per-ray formulation).
//
// Both kernels take 16 time samples [jbase, jbase + 16) per launch.
#include <cuda_runtime.h>

#include <algorithm>

#include "rectv_internal.cuh"
#include "usfft_common.cuh"

namespace rectv {

namespace {

constexpr int kT = 16;
constexpr int kFW = kT + 2 * kR;   // footprint side (24)
constexpr int kCells = kFW * kFW;  // 576
constexpr int kChunks = 8;         // 16-byte chunks of a cell: time samples (2i, 2i+1), complex

// ---- forward ----
constexpr int kFThr = 256;
constexpr int kFCap = 128;  // positions per forward item

constexpr int kWt = 5 * kTaps;  // weights per position (odd row pitch: the four positions of a warp on distinct banks)

struct FwdSmem {
    float4 fp[kCells * kChunks];  // footprint of 16 time samples, cell-major; chunk i of cell c at
                                  // slot (i + 2 (c & 3)) & 7
    // per position: [0,9) (-1)^b w_b of the x taps, [9,18) their derivatives
    // along x, [18,27) (-1)^a w_a of the y taps times the stencil origin's
    // fftshift sign, [27,36) those times cos, [36,45) minus sin times their
    // derivatives along y (cos, sin of the direction): S_perp's row weights
    float wt[kFCap][kWt];
    int org[kFCap];               // footprint cell of the stencil origin
    int pid[kFCap];               // d*n + q, -1: none
};

// ---- adjoint ----
constexpr int kAThr = 256;             // two threads per cell of a tile (8 time samples each), one slice per block
constexpr int kABlk = 16;              // 4x4-cell blocks of a tile: block b = rows 4 (b >> 2) .. + 3, columns 4 (b & 3) .. + 3
constexpr int kATab = 128;             // entries per table (host table builder)
constexpr int kAMaxSeg = 16;           // directions per table (host table builder)
constexpr int kAInfo = dir_adj_info_words(kAMaxSeg);
constexpr int kMThr = 256;             // positions per k_adj_mix block
constexpr int kMRays = 32;             // rays per staged chunk of k_adj_mix
constexpr int kMFly = 4;               // row loads in flight per thread of k_adj_mix

struct AdjSmem {
    AdjRec rec[2][kATab];                  // geometry records of this table and the next
    uint32_t info[2][kAInfo];              // their direction segmentation
    float4 e[2][kATab][2 * kChunks];       // [buffer][entry]: E_j in [0, 8), E_perp_j in [8, 16)
    int4 meta[2];                          // (tile, slice, entries or -1: none, last table of its unit)
};

__device__ __forceinline__ uint32_t saddr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void cp_async16(void *dst, const void *src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(saddr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// conj(a) b
__device__ __forceinline__ float2 cmulc(float2 a, float2 b) {
    return make_float2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}

}  // namespace

// ---------------------------------------------------------------------------
// Forward: one block (256 threads) per (work item, slices); an item is at
// most 128 positions whose stencils start in one 16x16 tile of the
// oversampled grid.  Per slice the tile's 24x24-cell footprint of 16 time
// samples is copied (coalesced loads, cell-major stores) from the halo-padded
// spectra (tiles right of the Nyquist column read the mirrored cells and
// conjugate), then eight lanes per position (two time samples each) sum the
// 81 taps, and mix the position's rays: each lane forms its two time
// samples' share of all eight rays of a round, the eight lanes add their
// shares by recursive halving (14 shuffles) and lane i keeps ray i.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kFThr, 2)
    k_gather_dir(float2 *__restrict__ rows, const float2 *__restrict__ spec, const uint32_t *__restrict__ pos,
                 const int4 *__restrict__ items, const float2 *__restrict__ dsincos,
                 const int *__restrict__ ray_start, const uint32_t *__restrict__ rays,
                 const float *__restrict__ tau, const float2 *__restrict__ kmat, const float2 *__restrict__ shiftf,
                 UsGeo g, int zb, int jbase, int accumulate, int *__restrict__ err) {
    extern __shared__ __align__(16) unsigned char dir_fwd_smem[];
    FwdSmem &sm = *reinterpret_cast<FwdSmem *>(dir_fwd_smem);
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int4 it = items[blockIdx.x];
    const int z0 = blockIdx.y * g.zper, z1 = min(zb, z0 + g.zper);
    const int tyi = it.x / g.NT, txi = it.x - tyi * g.NT;
    const int cnt = min(it.z, kFCap);
    const bool mirrored = txi * kT > g.n + 2;
    const int KY0 = tyi * kT - kR, KX0 = txi * kT - kR;  // footprint cell (0, 0) in the periodic spectrum

    // ---- the item's positions (the same for every slice) ----
    // derivative of a tap weight exp(-pi^2/mu d^2) along the position, per
    // grid cell: c1 d w, c1 = 2 (pi^2/mu) / (2n)
    const float c1 = 2.f * g.wexp / g.tn;
    for (int e = tid; e < kFCap; e += kFThr) {
        int id = -1, org = 0;
        float *wt = sm.wt[e];
        if (e < cnt) {
            const uint32_t u = __ldg(pos + it.y + e);
            const int d = u / (uint32_t)g.n, q = u - d * g.n;
            const float2 sc = __ldg(dsincos + d);
            float x0, y0;
            int fx, fy;
            sample_pos(q, sc, g, x0, y0, fx, fy);
            const int lx0 = g.n + fx - txi * kT, ly0 = g.n + fy - tyi * kT;
            if (lx0 < 0 || lx0 >= kT || ly0 < 0 || ly0 >= kT) {  // host/device bin disagreement
                atomicAdd(err, 1);
            } else {
                id = (int)u;
                org = ly0 * kFW + lx0;
                const float sgn = ((lx0 + ly0) & 1) ? -1.f : 1.f;
#pragma unroll
                for (int b = 0; b < kTaps; ++b) {
                    const float dx = (float)(fx - kR + b) * g.inv2n - x0, dy = (float)(fy - kR + b) * g.inv2n - y0;
                    const float a = tap_weight(fx, b, x0, g), c = tap_weight(fy, b, y0, g) * sgn;
                    const float sb = (b & 1) ? -1.f : 1.f;
                    wt[b] = sb * a;
                    wt[kTaps + b] = sb * c1 * dx * a;
                    wt[2 * kTaps + b] = sb * c;
                    wt[3 * kTaps + b] = sb * c * sc.y;
                    wt[4 * kTaps + b] = -sb * c1 * dy * c * sc.x;
                }
            }
        }
        if (id < 0)
            for (int b = 0; b < kWt; ++b) wt[b] = 0.f;
        sm.pid[e] = id;
        sm.org[e] = org;
    }

    const int ngroups = (cnt + 3) / 4;  // four positions per warp
    const int pi = lane >> 3, ci = lane & 7;
    const int fc = lane & 3, fj = lane >> 2;  // footprint copies: cell of four, time sample of eight
    const int j0 = jbase + 2 * ci;      // this lane's time samples j0, j0 + 1
    for (int z = z0; z < z1; ++z) {
        // ---- footprint of slice z: lane = (cell cl of four, time sample jj of
        // eight), warp w copies rows w, w + 8, w + 16: a half-warp writes four
        // cells x four time samples on distinct banks, a warp reads eight
        // 32-byte runs ----
        // (all 36 loads of a thread in flight, then the stores)
        const float2 *simg = spec + ((long long)z * g.m + jbase) * g.img_fwd;
        float2 fv[2][kFW / 8][kFW / 4];
#pragma unroll
        for (int jh = 0; jh < 2; ++jh) {
            const int j = 8 * jh + fj;
            const float2 *sj = simg + (long long)j * g.img_fwd;
#pragma unroll
            for (int rr = 0; rr < kFW / 8; ++rr) {
                const int KY = KY0 + wid + 8 * rr;
                const float2 *srow = sj + (long long)((mirrored ? g.P - KY : KY) + kHalo) * g.qp;
#pragma unroll
                for (int cq = 0; cq < kFW / 4; ++cq) {
                    const int KX = KX0 + 4 * cq + fc;
                    fv[jh][rr][cq] = (jbase + j < g.m) ? __ldg(srow + (mirrored ? g.P - KX : KX) + kHalo)
                                                       : make_float2(0.f, 0.f);
                }
            }
        }
#pragma unroll
        for (int jh = 0; jh < 2; ++jh) {
            const int j = 8 * jh + fj;
#pragma unroll
            for (int rr = 0; rr < kFW / 8; ++rr) {
                const int row = wid + 8 * rr;
                float2 *drow = reinterpret_cast<float2 *>(sm.fp) + (row * kFW + fc) * 16 + ((j + 4 * fc) & 15);
#pragma unroll
                for (int cq = 0; cq < kFW / 4; ++cq) drow[64 * cq] = fv[jh][rr][cq];
            }
        }
        __syncthreads();

        for (int gi = wid; gi < ngroups; gi += kFThr / 32) {
            const int e = 4 * gi + pi;
            const int id = sm.pid[e];
            const int org = sm.org[e];
            const int lx0 = org % kFW;
            // four base pointers (one per rotation of the column's chunks): every
            // tap is then a load at a constant offset from one of them
            const float4 *fq[4];
#pragma unroll
            for (int bq = 0; bq < 4; ++bq) fq[bq] = sm.fp + org * kChunks + ((ci + 2 * ((lx0 + bq) & 3)) & 7);
            const float *wt = sm.wt[e];
            float wx[kTaps], wxd[kTaps];
#pragma unroll
            for (int b = 0; b < kTaps; ++b) {
                wx[b] = wt[b];
                wxd[b] = wt[kTaps + b];
            }
            // ---- S_j and S_perp_j of this lane's two time samples: 81 taps ----
            float2 s0 = make_float2(0.f, 0.f), s1 = make_float2(0.f, 0.f);
            float2 p0 = make_float2(0.f, 0.f), p1 = make_float2(0.f, 0.f);
#pragma unroll
            for (int a = 0; a < kTaps; ++a) {
                float2 r0 = make_float2(0.f, 0.f), r1 = make_float2(0.f, 0.f);
                float2 d0 = make_float2(0.f, 0.f), d1 = make_float2(0.f, 0.f);
#pragma unroll
                for (int b = 0; b < kTaps; ++b) {
                    const float4 f = fq[b & 3][(a * kFW + b) * kChunks];
                    r0 = ffma2(make_float2(wx[b], wx[b]), make_float2(f.x, f.y), r0);
                    r1 = ffma2(make_float2(wx[b], wx[b]), make_float2(f.z, f.w), r1);
                    d0 = ffma2(make_float2(wxd[b], wxd[b]), make_float2(f.x, f.y), d0);
                    d1 = ffma2(make_float2(wxd[b], wxd[b]), make_float2(f.z, f.w), d1);
                }
                const float w = wt[2 * kTaps + a], wc = wt[3 * kTaps + a], ws = wt[4 * kTaps + a];
                s0 = ffma2(make_float2(w, w), r0, s0);
                s1 = ffma2(make_float2(w, w), r1, s1);
                p0 = ffma2(make_float2(wc, wc), d0, ffma2(make_float2(ws, ws), r0, p0));
                p1 = ffma2(make_float2(wc, wc), d1, ffma2(make_float2(ws, ws), r1, p1));
            }
            if (mirrored) {  // the footprint held the conjugate-mirrored cells
                s0.y = -s0.y;
                s1.y = -s1.y;
                p0.y = -p0.y;
                p1.y = -p1.y;
            }
            // ---- rays of the position, eight per round ----
            int q = 0, rs = 0, nr = 0;
            if (id >= 0) {
                const int d = id / g.n;
                q = id - d * g.n;
                rs = __ldg(ray_start + d);
                nr = __ldg(ray_start + d + 1) - rs;
            }
            const float qp = __fdiv_rn((float)(q - g.n / 2), (float)g.n);
            const int rounds = __reduce_max_sync(0xffffffffu, (nr + 7) >> 3);
            for (int rd = 0; rd < rounds; ++rd) {
                // lane ci fetches ray 8 rd + ci of its position; the eight lanes share them by shuffles
                uint32_t rv = 0;
                float tv = 0.f;
                if (8 * rd + ci < nr) {
                    rv = __ldg(rays + rs + 8 * rd + ci);
                    tv = __ldg(tau + rs + 8 * rd + ci);
                }
                float v[16];
#pragma unroll
                for (int rr = 0; rr < 8; ++rr) {
                    const uint32_t rvr = __shfl_sync(0xffffffffu, rv, (lane & ~7) | rr);
                    const float tvr = __shfl_sync(0xffffffffu, tv, (lane & ~7) | rr);
                    float2 k0 = make_float2(0.f, 0.f), k1 = make_float2(0.f, 0.f);
                    float dl = 0.f;
                    if (8 * rd + rr < nr) {
                        const long long th = rvr & 0x7fffffffu;
                        dl = qp * tvr;  // this ray's offset across the direction
                        if (j0 < g.m) k0 = __ldg(kmat + th * g.m + j0);
                        if (j0 + 1 < g.m) k1 = __ldg(kmat + th * g.m + j0 + 1);
                    }
                    const float2 t0 = make_float2(fmaf(dl, p0.x, s0.x), fmaf(dl, p0.y, s0.y));
                    const float2 t1 = make_float2(fmaf(dl, p1.x, s1.x), fmaf(dl, p1.y, s1.y));
                    v[2 * rr] = k0.x * t0.x - k0.y * t0.y + k1.x * t1.x - k1.y * t1.y;
                    v[2 * rr + 1] = k0.x * t0.y + k0.y * t0.x + k1.x * t1.y + k1.y * t1.x;
                }
                // sum over the eight lanes of the position by recursive halving;
                // lane ci ends with ray 8 rd + ci
                float w8[8], w4[4], w2[2];
                const bool b4 = ci & 4, b2 = ci & 2, b1 = ci & 1;
#pragma unroll
                for (int t = 0; t < 8; ++t) {
                    const float send = b4 ? v[t] : v[8 + t];
                    const float keep = b4 ? v[8 + t] : v[t];
                    w8[t] = keep + __shfl_xor_sync(0xffffffffu, send, 4);
                }
#pragma unroll
                for (int t = 0; t < 4; ++t) {
                    const float send = b2 ? w8[t] : w8[4 + t];
                    const float keep = b2 ? w8[4 + t] : w8[t];
                    w4[t] = keep + __shfl_xor_sync(0xffffffffu, send, 2);
                }
#pragma unroll
                for (int t = 0; t < 2; ++t) {
                    const float send = b1 ? w4[t] : w4[2 + t];
                    const float keep = b1 ? w4[2 + t] : w4[t];
                    w2[t] = keep + __shfl_xor_sync(0xffffffffu, send, 1);
                }
                const int ri = 8 * rd + ci;
                if (ri < nr) {
                    const long long th = rv & 0x7fffffffu;
                    const int k = (rv >> 31) ? g.n - q : q;
                    const float2 sh = __ldg(shiftf + k);
                    const float cf = (k & 1) ? g.cw : -g.cw;  // (-1)^(k+1) (pi/mu)/n
                    float2 o = cmul(make_float2(w2[0], w2[1]), make_float2(sh.x * cf, sh.y * cf));
                    float2 *dst = rows + ((long long)z * g.ntheta + th) * g.n + k;
                    if (accumulate) {
                        const float2 p = *dst;
                        o.x += p.x;
                        o.y += p.y;
                    }
                    *dst = o;
                }
            }
        }
        __syncthreads();  // the footprint buffer is refilled for the next slice
    }
}

// ---------------------------------------------------------------------------
// Adjoint, step 1: E_j and E_perp_j of every position and slice (time
// samples [jbase, jbase + 16)), once per position: one block per (direction,
// slice, 256 positions), one thread per position; the direction's rays are
// taken 32 at a time with their K' rows staged in shared memory, in ray
// order.  Out: emix[((z ndir + d) n + q)] = 16 float4, E of time samples
// (2i, 2i+1) in [i], E_perp in [8 + i].  The blocks also clear the nzero
// float4 of the half planes the scatter adds into (the memory pipe is idle
// in this latency-bound kernel).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kMThr, 2)
    k_adj_mix(float4 *__restrict__ emix, const float2 *__restrict__ rowsc, const int *__restrict__ ray_start,
              const uint32_t *__restrict__ rays, const float *__restrict__ tau, const float2 *__restrict__ kmat,
              const float2 *__restrict__ shifta, UsGeo g, int ndir, int jbase, float4 *__restrict__ zero,
              long long nzero) {
    __shared__ float2 ks[kMRays][16];
    {
        const long long nthr = (long long)gridDim.x * gridDim.y * gridDim.z * kMThr;
        const long long t0 = (((long long)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x) * kMThr +
                             threadIdx.x;
        for (long long i = t0; i < nzero; i += nthr) zero[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    __shared__ uint32_t rvs[kMRays];
    __shared__ float tvs[kMRays];
    const int d = blockIdx.x, z = blockIdx.y;
    const int q = blockIdx.z * kMThr + threadIdx.x;
    const int hn = g.n / 2 + 1;
    const int rs = __ldg(ray_start + d), nr = __ldg(ray_start + d + 1) - rs;
    const float qp = __fdiv_rn((float)(q - g.n / 2), (float)g.n);
    float2 e[16], ep[16];
#pragma unroll
    for (int j = 0; j < 16; ++j) e[j] = ep[j] = make_float2(0.f, 0.f);
    for (int r0 = 0; r0 < nr; r0 += kMRays) {
        const int nc = min(kMRays, nr - r0);
        __syncthreads();  // the previous chunk's rows are consumed
        for (int i = threadIdx.x; i < nc * 16; i += kMThr) {
            const int r = i >> 4, j = i & 15;
            const long long th = __ldg(rays + rs + r0 + r) & 0x7fffffffu;
            ks[r][j] = (jbase + j < g.m) ? __ldg(kmat + th * g.m + jbase + j) : make_float2(0.f, 0.f);
        }
        for (int r = threadIdx.x; r < nc; r += kMThr) {
            rvs[r] = __ldg(rays + rs + r0 + r);
            tvs[r] = __ldg(tau + rs + r0 + r);
        }
        __syncthreads();
        if (q >= 1 && q < g.n) {
            // the row factor of the two orientations: (-1)^(k+1) shiftadj(k) (pi/mu)/n, k = q or n - q
            const int kq = q, ko = g.n - q;
            const float2 shq = __ldg(shifta + kq), sho = __ldg(shifta + ko);
            const float cq = (kq & 1) ? g.cw : -g.cw, co = (ko & 1) ? g.cw : -g.cw;
            const float2 fq = make_float2(shq.x * cq, shq.y * cq), fo = make_float2(sho.x * co, sho.y * co);
            for (int r0c = 0; r0c < nc; r0c += kMFly) {
                // the row values of kMFly rays in flight together
                float2 R[kMFly];
#pragma unroll
                for (int i = 0; i < kMFly; ++i) {
                    R[i] = make_float2(0.f, 0.f);
                    if (r0c + i < nc) {
                        const uint32_t rv = rvs[r0c + i];
                        const long long th = rv & 0x7fffffffu;
                        const int k = (rv >> 31) ? ko : kq;
                        R[i] = __ldg(rowsc + ((long long)z * g.ntheta + th) * hn + (k <= g.n / 2 ? k : g.n - k));
                        if (k > g.n / 2) R[i].y = -R[i].y;  // the other half of the real row's spectrum
                    }
                }
#pragma unroll
                for (int i = 0; i < kMFly; ++i) {
                    if (r0c + i >= nc) break;
                    const uint32_t rv = rvs[r0c + i];
                    const float2 er = cmul(R[i], (rv >> 31) ? fo : fq);
                    const float dl = qp * tvs[r0c + i];  // this ray's offset across the direction
#pragma unroll
                    for (int j = 0; j < 16; ++j) {
                        const float2 a = cmulc(ks[r0c + i][j], er);
                        e[j].x += a.x;
                        e[j].y += a.y;
                        ep[j].x = fmaf(dl, a.x, ep[j].x);
                        ep[j].y = fmaf(dl, a.y, ep[j].y);
                    }
                }
            }
        }
    }
    if (q >= 1 && q < g.n) {
        float4 *o = emix + (((long long)z * ndir + d) * g.n + q) * 16;
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            o[i] = make_float4(e[2 * i].x, e[2 * i].y, e[2 * i + 1].x, e[2 * i + 1].y);
            o[8 + i] = make_float4(ep[2 * i].x, ep[2 * i].y, ep[2 * i + 1].x, ep[2 * i + 1].y);
        }
    }
}

// ---------------------------------------------------------------------------
// Adjoint, step 2: persistent blocks of 256 threads, two per SM, take (tile,
// slice) units round-robin (slices fastest, so that blocks in flight share
// their tiles' records in L2).  The 16x16 tile is cut into sixteen 4x4-cell
// blocks; a warp owns blocks w and 15 - w, its lane (h, cell) the cell of
// each block and the time samples [8h, 8h + 8).  A 9x9 stencil covers 56 %
// of the cells of the 4x4 blocks it touches (42 % of 4x8 blocks, 34 % of
// 2x16 rows), and two lanes per cell halve the E loads and packed FMAs a
// lane issues per entry.  A tile's entries (positions whose stencil touches
// it, direction-major) come in tables of at most 128 entries and 16
// directions, with the geometry records of the per-ray scatter (x and y
// weight rows over the tile, k_adj_records_dir) and per direction and block
// the entries that touch the block (k_adj_tabinfo_dir).  A copy cursor
// brings each table in (cp.async) while the table before it is processed:
// records and segmentation at its start, the entries' E, E_perp after its
// sums (their position ids have arrived by then), and the table's (tile,
// slice, entries) into shared memory beside them, so the sums wait on no
// global load.  Per table every cell adds
// w E_j + w_perp E_perp_j of the entries touching its block (FP32, entry
// order: reproducible).  The unit's sums go into the Hermitian half planes
// of the C2R inverse as in k_scatter_tc.
// ---------------------------------------------------------------------------
namespace {

// acc += sum over entries [e0, e1) of w E + w_perp E_perp for time samples
// [8h, 8h + 8) of cell (cx, cy); Eh = the entries' E with the lane's offset
__device__ __forceinline__ void dir_cell_sums(float (&acc)[16], const AdjRec *__restrict__ rec,
                                              const float4 *__restrict__ Eh, int e0, int e1, int cx, int cy,
                                              float bxy) {
#pragma unroll 2
    for (int e = e0; e < e1; ++e) {
        const float w = rec[e].wx[cx] * rec[e].wy[cy];
        const float wp = w * (rec[e].sf.x + bxy);
        const float4 *E = Eh + e * (2 * kChunks);
        const float2 ww = make_float2(w, w), pp = make_float2(wp, wp);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const float4 f = E[i], fp = E[kChunks + i];
            float2 a0 = ffma2(ww, make_float2(f.x, f.y), make_float2(acc[4 * i], acc[4 * i + 1]));
            float2 a1 = ffma2(ww, make_float2(f.z, f.w), make_float2(acc[4 * i + 2], acc[4 * i + 3]));
            a0 = ffma2(pp, make_float2(fp.x, fp.y), a0);
            a1 = ffma2(pp, make_float2(fp.z, fp.w), a1);
            acc[4 * i] = a0.x;
            acc[4 * i + 1] = a0.y;
            acc[4 * i + 2] = a1.x;
            acc[4 * i + 3] = a1.y;
        }
    }
}

// the Hermitian half-plane adds of one cell's sums (time samples [jb, jb + 8))
__device__ __forceinline__ void dir_cell_store(float2 *__restrict__ spec, const float (&acc)[16], int KX, int KY,
                                               const UsGeo &g, int z, int jb) {
    const int P = g.P;
    if (KY >= P || KX >= P) return;
    const int half = P / 2, hp = g.hpitch;
    const long long img_half = (long long)P * hp;
    const float sg = ((KX + KY) & 1) ? -0.5f : 0.5f;
    const bool here = KX <= half, mirror = KX >= half || KX == 0;
    const long long o1 = (long long)KY * hp + KX;
    const long long o2 = (long long)((P - KY) % P) * hp + (P - KX) % P;
    float2 *dst = spec + ((long long)z * g.m + jb) * img_half;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        if (jb + j >= g.m) break;
        const float2 v = make_float2(sg * acc[2 * j], sg * acc[2 * j + 1]);
        float2 *d = dst + (long long)j * img_half;
        if (here) atomicAdd(d + o1, v);
        if (mirror) atomicAdd(d + o2, make_float2(v.x, -v.y));
    }
}

}  // namespace

__global__ void __launch_bounds__(kAThr, 2)
    k_scatter_dir(const float4 *__restrict__ emix, float2 *__restrict__ spec, const AdjRec *__restrict__ recs,
                  const uint32_t *__restrict__ pts, const int4 *__restrict__ items, const int4 *__restrict__ tabs,
                  const int *__restrict__ tab_base, const uint32_t *__restrict__ info, UsGeo g, int ndir, int zb,
                  int nunits, int jbase) {
    extern __shared__ __align__(16) unsigned char dir_adj_smem[];
    AdjSmem &sm = *reinterpret_cast<AdjSmem *>(dir_adj_smem);
    const int tid = threadIdx.x, wid = tid >> 5, lane = tid & 31;
    // this thread's cells: (rx, ry) of blocks b0 = wid and b1 = 15 - wid, time samples [8h, 8h + 8)
    const int h = lane >> 4, rx = lane & 3, ry = (lane >> 2) & 3;
    const int b0 = wid, b1 = kABlk - 1 - wid;
    const int cx0 = 4 * (b0 & 3) + rx, cy0 = 4 * (b0 >> 2) + ry;
    const int cx1 = 4 * (b1 & 3) + rx, cy1 = 4 * (b1 >> 2) + ry;

    // Copy cursor: the tables in consumption order (units u = blockIdx.x,
    // + gridDim.x, ...; the tables of a unit in order).  The descriptor of the
    // table to copy next and the table range and tile of the unit after the
    // cursor's are loaded one step ahead, and a table's E, E_perp copies are
    // issued after the sums of the table before it, so that no load latency
    // sits in front of a copy.
    const int pe = tid >> 1, pc0 = (tid & 1) * 8;  // entry and half of its 16 chunks this thread copies
    int fu = blockIdx.x, fti = 0, ftb1 = 0, ftile = 0, ntb0 = 0, ntb1 = 0, ntile = 0;
    int4 fdesc = make_int4(0, 0, 0, 0);  // (first entry, count, word offset, words)
    int pz = 0, pcnt = 0;                // the E copy still to issue: slice, entries
    uint32_t ppid = 0;                   // and this thread's position d*n + q
    if (fu < nunits) {
        const int item = fu / zb;
        fti = __ldg(tab_base + item);
        ftb1 = __ldg(tab_base + item + 1);
        ftile = __ldg(items + item).x;
        fdesc = __ldg(tabs + fti);
    }
    if (fu + (int)gridDim.x < nunits) {
        const int item = (fu + (int)gridDim.x) / zb;
        ntb0 = __ldg(tab_base + item);
        ntb1 = __ldg(tab_base + item + 1);
        ntile = __ldg(items + item).x;
    }
    // records, segmentation and the table's (tile, slice, entries, last of its
    // unit) into slot; entries -1: no table left
    auto fetch_a = [&](int slot) {
        if (fu < nunits) {
            const int cnt = min(fdesc.y, kATab), nw = min(fdesc.w, kAInfo);
            const char *rs = reinterpret_cast<const char *>(recs + fdesc.x);
            char *rd = reinterpret_cast<char *>(sm.rec[slot]);
            constexpr int kRecChunks = (int)(sizeof(AdjRec) / 16);
            for (int c = tid; c < cnt * kRecChunks; c += kAThr) cp_async16(rd + 16 * c, rs + 16 * c);
            const char *is = reinterpret_cast<const char *>(info + fdesc.z);
            char *id = reinterpret_cast<char *>(sm.info[slot]);
            for (int c = tid; c < nw / 4; c += kAThr) cp_async16(id + 16 * c, is + 16 * c);
            pz = fu % zb;
            pcnt = cnt;
            ppid = pe < cnt ? __ldg(pts + fdesc.x + pe) : 0u;
            if (tid == 0) sm.meta[slot] = make_int4(ftile, pz, cnt, fti + 1 >= ftb1 ? 1 : 0);
            if (++fti >= ftb1) {  // the next unit: its range and tile were loaded one unit ago
                fu += gridDim.x;
                fti = ntb0;
                ftb1 = ntb1;
                ftile = ntile;
                const int nu = fu + (int)gridDim.x;
                if (nu < nunits) {
                    const int item = nu / zb;
                    ntb0 = __ldg(tab_base + item);
                    ntb1 = __ldg(tab_base + item + 1);
                    ntile = __ldg(items + item).x;
                }
            }
            if (fu < nunits) fdesc = __ldg(tabs + fti);
        } else {
            pcnt = 0;
            if (tid == 0) sm.meta[slot] = make_int4(0, 0, -1, 0);
        }
        cp_commit();
    };
    // E, E_perp of the table fetch_a last took (its position ids have arrived by now)
    auto fetch_b = [&](int slot) {
        if (pe < pcnt) {
            const float4 *src = emix + ((long long)pz * ndir * g.n + ppid) * 16 + pc0;
            float4 *dst = &sm.e[slot][pe][pc0];
#pragma unroll
            for (int c = 0; c < 8; ++c) cp_async16(dst + c, src + c);
        }
        cp_commit();
    };

    float acc0[16], acc1[16];  // F of the two cells: 8 time samples x (re, im)
#pragma unroll
    for (int i = 0; i < 16; ++i) acc0[i] = acc1[i] = 0.f;
    fetch_a(0);
    fetch_b(0);
    for (int buf = 0;; buf ^= 1) {
        fetch_a(buf ^ 1);  // the next table: that buffer was released by the last barrier
        cp_wait<1>();      // everything but that group: this table's copies
        __syncthreads();
        const int4 mt = sm.meta[buf];  // (tile, slice, entries, last table of the unit)
        if (mt.z < 0) break;
        const int cnt = mt.z;
        const AdjRec *rec = sm.rec[buf];
        const uint32_t *inf = sm.info[buf];
        const float4 *Eh = &sm.e[buf][0][4 * h];
        const int nseg = min(min((int)inf[0], cnt), kAMaxSeg);
        const uint16_t *segf = reinterpret_cast<const uint16_t *>(inf + 4 + kABlk * nseg);  // direction starts
        for (int s = 0; s < nseg; ++s) {
            const uint32_t lh0 = inf[4 + kABlk * s + b0], lh1 = inf[4 + kABlk * s + b1];
            const int e00 = (int)(lh0 & 0xffffu), e01 = min((int)(lh0 >> 16), cnt);
            const int e10 = (int)(lh1 & 0xffffu), e11 = min((int)(lh1 >> 16), cnt);
            if (e00 >= e01 && e10 >= e11) continue;
            // first-order weight w (A_p + B . (cx, cy)): B of the direction from its first record
            const AdjRec &r0 = rec[min((int)segf[s], cnt - 1)];
            const float bx = r0.sf.y, by = __int_as_float(r0.k);
            dir_cell_sums(acc0, rec, Eh, e00, e01, cx0, cy0, bx * (float)cx0 + by * (float)cy0);
            dir_cell_sums(acc1, rec, Eh, e10, e11, cx1, cy1, bx * (float)cx1 + by * (float)cy1);
        }
        fetch_b(buf ^ 1);
        __syncthreads();  // the records, segmentation and E of this buffer are free
        if (mt.w) {
            // ---- the adjoint only needs Re IFFT2(X) = C2R of the Hermitian part
            // H(k) = (X(k) + conj X(-k)) / 2 on the half plane kx <= n: each cell adds
            // X(k)/2 to H(k) and conj(X(k))/2 to H(-k) where they lie in the half
            // plane (at most two adds per H cell, onto zeros: the sum does not depend
            // on their order); the pre-IFFT fftshift sign is applied here ----
            const int tyi = mt.x / g.NT, txi = mt.x - tyi * g.NT;
            dir_cell_store(spec, acc0, txi * kT + cx0, tyi * kT + cy0, g, mt.y, jbase + 8 * h);
            dir_cell_store(spec, acc1, txi * kT + cx1, tyi * kT + cy1, g, mt.y, jbase + 8 * h);
#pragma unroll
            for (int i = 0; i < 16; ++i) acc0[i] = acc1[i] = 0.f;
        }
    }
    cp_wait<0>();  // the cursor's last (empty) groups
}

// ---------------------------------------------------------------------------
// Geometry records of the direction path's adjoint entries: those of
// k_adj_records (scatter_tc.cu) for the direction's representative
// positions, with the first-order weight's constants in place of the
// per-ray fields: at tile cell (cx, cy) the distance to the position along x
// is cx/(2n) + ax (and likewise y), so cos dw/dx w_y - sin w_x dw/dy =
// w (A + B . (cx, cy)) with A = c1 (cos ax - sin ay) in sf.x and
// B = c1/(2n) (cos, -sin) in sf.y and k (float bits), c1 = 2 (pi^2/mu)/(2n).
// thm holds the direction and the 4x4-cell blocks of the tile the stencil
// touches.  One block per work item, one thread per entry.
// ---------------------------------------------------------------------------
__global__ void k_adj_records_dir(AdjRec *__restrict__ recs, const uint32_t *__restrict__ pts,
                                  const int4 *__restrict__ items, const float2 *__restrict__ dsincos, UsGeo g) {
    const int4 it = items[blockIdx.x];
    const int tyi = it.x / g.NT, txi = it.x - tyi * g.NT;
    const int P = g.P, half = P / 2;
    const float c1 = 2.f * g.wexp / g.tn;
    for (int e = threadIdx.x; e < it.z; e += blockDim.x) {
        const uint32_t id = pts[it.y + e];
        const int d = id / (uint32_t)g.n;
        const int q = id - d * g.n;
        const float2 sc = dsincos[d];
        float x0, y0;
        int fx, fy;
        sample_pos(q, sc, g, x0, y0, fx, fy);
        int dx = g.n + fx - kR - txi * kT;
        int dy = g.n + fy - kR - tyi * kT;
        dx += (dx < -half) ? P : 0;
        dx -= (dx > half) ? P : 0;
        dy += (dy < -half) ? P : 0;
        dy -= (dy > half) ? P : 0;
        AdjRec r;
        int rows = 0, cols = 0;
#pragma unroll
        for (int c = 0; c < kT; ++c) {
            const int bx = c - dx, by = c - dy;
            const bool inx = (unsigned)bx < (unsigned)kTaps, iny = (unsigned)by < (unsigned)kTaps;
            r.wx[c] = inx ? tap_weight(fx, bx, x0, g) : 0.f;
            r.wy[c] = iny ? tap_weight(fy, by, y0, g) : 0.f;
            rows |= iny ? (1 << c) : 0;
            cols |= inx ? (1 << c) : 0;
        }
        // 4x4-cell blocks of k_scatter_dir the stencil touches (block b: rows
        // 4 (b >> 2) .. + 3, columns 4 (b & 3) .. + 3) as bit b
        int mask = 0;
#pragma unroll
        for (int b = 0; b < kABlk; ++b)
            if (((rows >> (4 * (b >> 2))) & 0xf) && ((cols >> (4 * (b & 3))) & 0xf)) mask |= 1 << b;
        r.thm = (d << 16) | mask;
        const float ax = (float)(fx - kR - dx) * g.inv2n - x0, ay = (float)(fy - kR - dy) * g.inv2n - y0;
        const float cb = c1 * g.inv2n;
        r.sf = make_float2(c1 * (sc.y * ax - sc.x * ay), cb * sc.y);
        r.k = __float_as_int(-cb * sc.x);
        recs[(long long)it.y + e] = r;
    }
}

void launch_adj_records_dir(AdjRec *recs, const GeoDev &gd, const UsGeo &g, cudaStream_t s) {
    if (gd.n_adj_items == 0) return;
    k_adj_records_dir<<<gd.n_adj_items, 256, 0, s>>>(recs, gd.adj_pts, gd.adj_items, gd.sincos, g);
    LAUNCH_CHECK("k_adj_records_dir");
}

// ---------------------------------------------------------------------------
// Segmentation of every direction-path adjoint table (geometry only, so
// computed once), in the layout of dir_adj_info_words: the directions (runs
// of equal thm >> 16, records are direction-major), their first rows, and per
// direction and 4x4-cell block the rows [lo, hi) from the first to the last
// entry whose stencil touches the block (found at the entries where a
// touching run starts or ends; rows in between that miss the block have
// zero weights there).  One block per table, one thread per entry.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kATab)
    k_adj_tabinfo_dir(const AdjRec *__restrict__ recs, const int4 *__restrict__ tabs, uint32_t *__restrict__ info) {
    __shared__ int seg_first[kAMaxSeg + 1];
    __shared__ int rlo[kABlk][kAMaxSeg], rhi[kABlk][kAMaxSeg];
    __shared__ int wsum[kATab / 32];
    const int4 tb = tabs[blockIdx.x];  // (first entry, count, word offset, words)
    const int ct = threadIdx.x, lane = ct & 31, w = ct >> 5, cnt = min(tb.y, kATab);
    int thm = 0, thp = 0, thn = 0;
    if (ct < cnt) {
        thm = recs[(long long)tb.x + ct].thm;
        if (ct > 0) thp = recs[(long long)tb.x + ct - 1].thm;
        if (ct + 1 < cnt) thn = recs[(long long)tb.x + ct + 1].thm;
    }
    const unsigned d = (unsigned)thm >> 16;
    const int flag = (ct < cnt && (ct == 0 || ((unsigned)thp >> 16) != d)) ? 1 : 0;
    int incl = flag;  // inclusive scan of the direction starts
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) wsum[w] = incl;
    for (int i = ct; i < kABlk * kAMaxSeg; i += kATab) {
        rlo[i / kAMaxSeg][i % kAMaxSeg] = kATab;
        rhi[i / kAMaxSeg][i % kAMaxSeg] = 0;
    }
    __syncthreads();
    int base = 0, nseg = 0;
#pragma unroll
    for (int i = 0; i < kATab / 32; ++i) {
        base += (i < w) ? wsum[i] : 0;
        nseg += wsum[i];
    }
    nseg = min(nseg, kAMaxSeg);  // the host's tables hold at most kAMaxSeg directions
    const int seg = incl + base - 1;
    if (ct < cnt && flag && seg < kAMaxSeg) seg_first[seg] = ct;
    if (ct == 0) seg_first[nseg] = cnt;
    __syncthreads();
    if (ct < cnt && seg < kAMaxSeg) {
        const int msk = thm & 0xffff;
        const int mprev = flag ? 0 : (thp & 0xffff);
        const bool last = ct + 1 == cnt || ((unsigned)thn >> 16) != d;
        const int mnext = last ? 0 : (thn & 0xffff);
#pragma unroll
        for (int b = 0; b < kABlk; ++b) {
            const int bit = 1 << b;
            if (msk & bit) {
                if (!(mprev & bit)) atomicMin(&rlo[b][seg], ct);
                if (!(mnext & bit)) atomicMax(&rhi[b][seg], ct + 1);
            }
        }
    }
    __syncthreads();
    uint32_t *out = info + tb.z;
    const int nw = min(dir_adj_info_words(nseg), tb.w);  // the host sized the slot from the same directions
    for (int i = ct; i < nw; i += kATab) {
        uint32_t v = 0;
        if (i == 0) {
            v = (uint32_t)nseg;
        } else if (i >= 4 && i < 4 + kABlk * nseg) {
            const int sg = (i - 4) / kABlk, b = (i - 4) % kABlk;
            v = (uint32_t)rlo[b][sg] | ((uint32_t)rhi[b][sg] << 16);
        } else if (i >= 4 + kABlk * nseg) {
            const int j = 2 * (i - 4 - kABlk * nseg);  // 16-bit direction starts j, j+1
            if (j <= nseg) v = (uint32_t)seg_first[j];
            if (j + 1 <= nseg) v |= (uint32_t)seg_first[j + 1] << 16;
        }
        out[i] = v;
    }
}

void launch_adj_tabinfo_dir(const GeoDev &gd, cudaStream_t s) {
    if (gd.n_adj_tabs == 0) return;
    k_adj_tabinfo_dir<<<gd.n_adj_tabs, kATab, 0, s>>>(gd.adj_recs, gd.adj_tabs, gd.adj_info);
    LAUNCH_CHECK("k_adj_tabinfo_dir");
}

void dir_prepare() {
    CUDA_CHECK(cudaFuncSetAttribute(k_gather_dir, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(FwdSmem)));
    CUDA_CHECK(cudaFuncSetAttribute(k_scatter_dir, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(AdjSmem)));
}

int dir_fwd_capacity() { return kFCap; }
int dir_adj_table_capacity() { return kATab; }
int dir_adj_table_dirs() { return kAMaxSeg; }
size_t dir_mix_bytes(int zb, int ndir, int n) { return (size_t)zb * ndir * n * 16 * sizeof(float4); }

void launch_gather_dir(float2 *rows, const float2 *spec, int zb, const GeoDev &gd, const UsGeo &g, int jbase,
                       int accumulate, cudaStream_t s) {
    if (gd.n_dfwd_items == 0) return;
    if (g.T != kT) throw Error(1, "tile size must be 16");
    if (g.zper < 1) throw Error(1, "slices per block must be positive");
    const dim3 gs(gd.n_dfwd_items, (zb + g.zper - 1) / g.zper);
    k_gather_dir<<<gs, kFThr, sizeof(FwdSmem), s>>>(rows, spec, gd.dfwd_pos, gd.dfwd_items, gd.sincos, gd.dray_start,
                                                     gd.drays, gd.dtau, gd.kmat, gd.shiftfwd, g, zb, jbase, accumulate,
                                                     gd.err);
    LAUNCH_CHECK("k_gather_dir");
}

void launch_scatter_dir(const float2 *rowsc, float2 *spec, int zb, const GeoDev &gd, const UsGeo &g, int jbase,
                        cudaStream_t s) {
    if (g.T != kT) throw Error(1, "tile size must be 16");
    if (!gd.adj_recs || !gd.adj_tabs || !gd.adj_info || !gd.demix) throw Error(1, "adjoint direction tables missing");
    const long long nunits = (long long)zb * gd.n_adj_busy;
    if (nunits == 0) return;
    if (nunits > 2147483647LL - 65536) throw Error(1, "adjoint grid too large");  // the cursor adds the grid size
    if (zb > gd.demix_slices) throw Error(1, "adjoint direction mixing buffer too small");
    const dim3 gm(gd.ndir, zb, (g.n + kMThr - 1) / kMThr);
    // the first group of time samples also clears the half planes of all of them
    const long long nzero = jbase == 0 ? (long long)zb * g.m * g.P * g.hpitch / 2 : 0;
    k_adj_mix<<<gm, kMThr, 0, s>>>(gd.demix, rowsc, gd.dray_start, gd.drays, gd.dtau, gd.kmat, gd.shiftadj, g, gd.ndir,
                                   jbase, reinterpret_cast<float4 *>(spec), nzero);
    LAUNCH_CHECK("k_adj_mix");
    static int nsm = 0;
    if (nsm == 0) {
        int dev = 0;
        CUDA_CHECK(cudaGetDevice(&dev));
        CUDA_CHECK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    }
    const int grid = (int)std::min<long long>(nunits, g.sc_grid > 0 ? g.sc_grid : 2 * nsm);
    k_scatter_dir<<<grid, kAThr, sizeof(AdjSmem), s>>>(gd.demix, spec, gd.adj_recs, gd.adj_pts, gd.adj_items,
                                                       gd.adj_tabs, gd.adj_tab_base, gd.adj_info, g, gd.ndir, zb,
                                                       (int)nunits, jbase);
    LAUNCH_CHECK("k_scatter_dir");
}

}  // namespace rectv
