// 4D total-variation and ADMM kernels (x, y, time, z) for sm_103a.
//
// The reference builds an extended copy of the chunk (extendf), writes the
// float4 gradient (gradf), then runs separate axpby passes and the divergence
// (kernels_operators.cuh:4-73, admm.cu:5-122).  Here the inner step
//   u <- u - 1/2 div( rho (G u - psi) + mu )          (admm.cu:85-95)
// is one kernel that forms each needed gradient component on the fly, and the
// end-of-iteration shrink / dual update / residual norms (admm.cu:101-117)
// are another.  The norms are reduced in float64 in a fixed order so the rho
// rule (rectv.cu:223-232) is deterministic.
//
// Chunk semantics (rectv.cu:161-173, extendf): chunk c covers slices
// [c nzp, (c+1) nzp); the slice below/above a chunk is read from the previous
// outer iterate u_old (never the one being updated) and at the volume ends the
// border value is replicated.  Each chunk owns a dual grid of
// (n+1)^2 (m+1)(nzp+1) points whose point q sees voxel q-1 (clamped).
#include <cuda_runtime.h>

#include "rectv_internal.cuh"

namespace rectv {

namespace {

__device__ __forceinline__ int clampi(int a, int lo, int hi) { return a < lo ? lo : (a > hi ? hi : a); }

__device__ __forceinline__ void prefetch_l2(const void *p) {
    asm volatile("prefetch.global.L2 [%0];\n" ::"l"(p));
}

template <int NW>
__device__ __forceinline__ void block_reduce3(double a, double b, double c, double *out) {
    __shared__ double sh[3][NW];
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        b += __shfl_down_sync(0xffffffffu, b, o);
        c += __shfl_down_sync(0xffffffffu, c, o);
    }
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;  // 2D blocks
    const int lane = tid & 31, w = tid >> 5;
    if (lane == 0) {
        sh[0][w] = a;
        sh[1][w] = b;
        sh[2][w] = c;
    }
    __syncthreads();
    if (tid == 0) {
        double s0 = 0, s1 = 0, s2 = 0;
        for (int i = 0; i < NW; ++i) {
            s0 += sh[0][i];
            s1 += sh[1][i];
            s2 += sh[2][i];
        }
        out[0] = s0;
        out[1] = s1;
        out[2] = s2;
    }
}

}  // namespace

// ---------------------------------------------------------------------------
// Fused inner step (gradient, lin4, divergent of admm.cu:85-95 with tau=-0.5):
//   u_out(v) = u_in(v) + tau sd sum_d [h_d(q-e_d) - h_d(q)],  q = v+1,
//   h = rho (G u_in - psi) + mu = rho G u_in + w,  w = mu - rho psi.
// psi, mu and rho change only at the end of an outer iteration, so the first
// inner step (MODE 1) reads psi and mu and also stores w for every dual point
// the step reads, and the later ones (MODE 2) read w alone (half the dual
// bytes); MODE 0 reads psi and mu only.
// One thread per (x, y, slice), marching along t: h_t(q - e_t) is the previous
// time point's h_t(q), kept in a register, and the loads of time point t+1
// are issued before t is computed.  Blocks of 256 x-voxels; the grid runs
// over (x blocks, slices, rows) in that order, so the blocks that read a
// block's z-1 and y-1 dual neighbours run at the same time (L2 hits rather
// than second HBM reads).
// ---------------------------------------------------------------------------
template <int MODE>
__global__ void __launch_bounds__(256, MODE == 2 ? 4 : 3)  // MODE 2 loads less: 32 warps per SM
    k_graddiv(const float *__restrict__ uin, const float *__restrict__ uold, float *__restrict__ uout,
              const float *__restrict__ psi, const float *__restrict__ mu, float *__restrict__ w,
              const float *__restrict__ rhop, TvGeo t, int c0, int nch_total, float tau) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int zr = blockIdx.y;
    const int y = blockIdx.z;
    if (x >= t.n) return;
    const int n = t.n, m = t.m, nzp = t.nzp;
    const int c = c0 + zr / nzp, zl = zr % nzp;
    const long long slab = t.vol_slab, nn = (long long)n * n;
    const long long v0 = ((long long)c * nzp + zl) * slab + (long long)y * n + x;  // voxel (x, y, t = 0)
    const float *u = uin + v0;
    // z neighbours: inside the chunk, else the previous outer iterate, else replicated
    const float *uzp = (zl < nzp - 1) ? uin + v0 + slab : ((c < nch_total - 1) ? uold + v0 + slab : u);
    const float *uzm = (zl > 0) ? uin + v0 - slab : ((c > 0) ? uold + v0 - slab : u);
    const int dxp = x < n - 1 ? 1 : 0, dxm = x > 0 ? 1 : 0;
    const int dyp = y < n - 1 ? n : 0, dym = y > 0 ? n : 0;
    const float rho = *rhop;
    const long long sx = 1, sy = n + 1, st = (long long)(n + 1) * (n + 1), sz = st * (m + 1);
    const long long cs = t.comp_stride;
    const long long q0 = (long long)c * t.gp + (zl + 1) * sz + st + (y + 1) * sy + (x + 1);  // q of t = 0
    const float sg = t.sg, sgt = t.sg * t.lambda1;
    // a[]: u at x+1, x-1, y+1, y-1, z+1, z-1, t+1; then the dual values: at q
    // (4 components) and of component x at q-sx, y at q-sy, z at q-sz, as
    // (psi, mu) pairs (MODE 0, 1: a[7..10] psi, a[11..14] mu, a[15..20]
    // psi/mu pairs) or w alone (MODE 2: a[7..10] w, a[15], a[17], a[19])
    auto load = [&](int tt, float(&a)[21]) {
        const long long o = (long long)tt * nn;
        const long long q = q0 + (long long)tt * st;
        a[0] = u[o + dxp];
        a[1] = u[o - dxm];
        a[2] = u[o + dyp];
        a[3] = u[o - dym];
        a[4] = uzp[o];
        a[5] = uzm[o];
        a[6] = u[o + (tt < m - 1 ? nn : 0)];
        if constexpr (MODE == 2) {
#pragma unroll
            for (int i = 0; i < 4; ++i) a[7 + i] = w[i * cs + q];
            a[15] = w[q - sx];
            a[17] = w[cs + q - sy];
            a[19] = w[3 * cs + q - sz];
        } else {
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                a[7 + i] = psi[i * cs + q];
                a[11 + i] = mu[i * cs + q];
            }
            a[15] = psi[q - sx];
            a[16] = mu[q - sx];
            a[17] = psi[cs + q - sy];
            a[18] = mu[cs + q - sy];
            a[19] = psi[3 * cs + q - sz];
            a[20] = mu[3 * cs + q - sz];
        }
    };
    // h of one component from the gradient term g and the dual values
    auto hval = [&](float g, const float(&a)[21], int ip, int im) {
        if constexpr (MODE == 2)
            return rho * g + a[ip];
        else
            return rho * (g - a[ip]) + a[im];
    };
    float cur[21];
    load(0, cur);
    float f0 = u[0];
    // h_t at q - st for t = 0: the clamped backward difference is zero
    float hmt;
    if constexpr (MODE == 2) {
        hmt = rho * (sgt * (f0 - f0)) + w[2 * cs + q0 - st];
    } else {
        const float p0 = psi[2 * cs + q0 - st], m0 = mu[2 * cs + q0 - st];
        hmt = rho * (sgt * (f0 - f0) - p0) + m0;
        if constexpr (MODE == 1) w[2 * cs + q0 - st] = m0 - rho * p0;
    }
    const float *wpf = w + q0 + 3 * st;  // MODE 2: w of time point tt + 3
    for (int tt = 0; tt < m; ++tt) {
        float nxt[21];
        if constexpr (MODE == 2) {
            // the dual lines only this thread's column brings from HBM (its own
            // w, 16 of the 20 new bytes per voxel; the neighbours' are other
            // threads' own), into L2 two time points before load() asks for
            // them: registers hold only one point ahead
            if (tt + 3 < m) {
#pragma unroll
                for (int i = 0; i < 4; ++i) prefetch_l2(wpf + i * cs);
            }
            wpf += st;
        }
        if (tt + 1 < m) load(tt + 1, nxt);
        if constexpr (MODE == 1) {  // w at q, and at the lower boundary planes this voxel reads
            const long long q = q0 + (long long)tt * st;
#pragma unroll
            for (int i = 0; i < 4; ++i) w[i * cs + q] = cur[11 + i] - rho * cur[7 + i];
            if (x == 0) w[q - sx] = cur[16] - rho * cur[15];
            if (y == 0) w[cs + q - sy] = cur[18] - rho * cur[17];
            if (zl == 0) w[3 * cs + q - sz] = cur[20] - rho * cur[19];
        }
        float d;
        {  // x
            const float hq = hval(sg * (cur[0] - f0), cur, 7, 11);
            const float hm = hval(sg * (f0 - cur[1]), cur, 15, 16);
            d = hm - hq;
        }
        {  // y
            const float hq = hval(sg * (cur[2] - f0), cur, 8, 12);
            const float hm = hval(sg * (f0 - cur[3]), cur, 17, 18);
            d += hm - hq;
        }
        {  // t (scaled by lambda1 in both gradient and divergence)
            const float hq = hval(sgt * (cur[6] - f0), cur, 9, 13);
            d += t.lambda1 * (hmt - hq);
            hmt = hq;
        }
        {  // z
            const float hq = hval(sg * (cur[4] - f0), cur, 10, 14);
            const float hm = hval(sg * (f0 - cur[5]), cur, 19, 20);
            d += hm - hq;
        }
        uout[v0 + (long long)tt * nn] = f0 + tau * t.sd * d;
        f0 = cur[6];  // u at t+1
        if (tt + 1 < m) {
#pragma unroll
            for (int i = 0; i < 21; ++i) cur[i] = nxt[i];
        }
    }
}

void launch_graddiv(const float *u_in, const float *u_old, float *u_out, const float *psi,
                    const float *mu, float *w, int mode, const float *rho, int c0, int nchunks_total,
                    const TvGeo &t, cudaStream_t s) {
    dim3 bs(256, 1), gs((t.n + 255) / 256, t.nchunks * t.nzp, t.n);
    if (gs.y > 65535u || gs.z > 65535u) throw Error(1, "graddiv: grid too large");
    if (mode != 0 && !w) throw Error(1, "graddiv: no w buffer");
    if (mode == 1)
        k_graddiv<1><<<gs, bs, 0, s>>>(u_in, u_old, u_out, psi, mu, w, rho, t, c0, nchunks_total, -0.5f);
    else if (mode == 2)
        k_graddiv<2><<<gs, bs, 0, s>>>(u_in, u_old, u_out, psi, mu, w, rho, t, c0, nchunks_total, -0.5f);
    else
        k_graddiv<0><<<gs, bs, 0, s>>>(u_in, u_old, u_out, psi, mu, w, rho, t, c0, nchunks_total, -0.5f);
    LAUNCH_CHECK("k_graddiv");
}

// ---------------------------------------------------------------------------
// End of outer iteration for one chunk (admm.cu:101-117):
//   h = G u_cur, ho = G u_old (the reference's h2stored),
//   psi = shrink(h + mu/rho, lambda0/rho), mu += rho h - rho psi,
//   sums of |h-psi|^2, |ho-h|^2 and, for q >= 1, (u_cur-u_old)^2.
// One thread per (qx, qy, qz) marching along qt; the squares along its qt
// column are summed in FP32 (at most m+1 = 17 terms for m = 16) and the
// thread sums are accumulated in FP64 in a fixed order; one FP64 partial
// triple per block.  Blocks of 32x8 over (qx, qy), grid.z over (chunk, qz).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256, 4)
    k_shrink(const float *__restrict__ ucur, const float *__restrict__ uold, float *__restrict__ psi,
             float *__restrict__ mu, const float *__restrict__ rhop, float lambda0, TvGeo t, int c0,
             int nch_total, double *__restrict__ partials) {
    const int qx = blockIdx.x * blockDim.x + threadIdx.x;
    const int qy = blockIdx.y * blockDim.y + threadIdx.y;
    const int n = t.n, m = t.m, nzp = t.nzp;
    const int qz = blockIdx.z % (nzp + 1);
    const int c = c0 + blockIdx.z / (nzp + 1);
    float a0 = 0.f, a1 = 0.f, a2 = 0.f;
    if (qx <= n && qy <= n) {
        const long long slab = t.vol_slab, nn = (long long)n * n;
        const long long zc = (long long)c * nzp;
        // extended-chunk slabs at z0 = qz-1 and z1 = qz (extendf, kernels_operators.cuh:14-19)
        auto slab_of = [&](const float *u, int zl) -> const float * {
            if (zl < 0) return (c > 0) ? uold + (zc - 1) * slab : u + zc * slab;
            if (zl >= nzp) return (c < nch_total - 1) ? uold + (zc + nzp) * slab : u + (zc + nzp - 1) * slab;
            return u + (zc + zl) * slab;
        };
        const float *c0p = slab_of(ucur, qz - 1), *c1p = slab_of(ucur, qz);
        const float *o0p = slab_of(uold, qz - 1), *o1p = slab_of(uold, qz);
        const int x0 = clampi(qx - 1, 0, n - 1), x1 = clampi(qx, 0, n - 1);
        const int y0 = clampi(qy - 1, 0, n - 1), y1 = clampi(qy, 0, n - 1);
        const long long p00 = (long long)y0 * n + x0, px = (long long)y0 * n + x1, py = (long long)y1 * n + x0;
        const bool inner_xyz = (qx >= 1 && qy >= 1 && qz >= 1);
        const float sg = t.sg, sgt = t.sg * t.lambda1;
        const float rho = *rhop;
        const float thr = lambda0 / rho, rinv = 1.0f / rho;
        const long long cs = t.comp_stride;
        long long q = (long long)c * t.gp + ((long long)qz * (m + 1)) * (n + 1) * (n + 1) + (long long)qy * (n + 1) + qx;
        const long long st = (long long)(n + 1) * (n + 1);
        float fc = c0p[p00], fo = o0p[p00];  // values at (x0, y0, t0 = clamp(qt-1) = 0, z0)
        // loads of time point qt + 1 are issued before qt is computed and
        // stored (two time points of loads in flight per thread)
        float lu[8], lm[4];
        auto load = [&](int qt, long long qq) {
            const long long o0 = (long long)(qt > 0 ? qt - 1 : 0) * nn;  // t0 = clamp(qt-1)
            const long long o1 = (long long)(qt < m ? qt : m - 1) * nn;  // t1 = clamp(qt)
            lu[0] = c0p[o0 + px];
            lu[1] = c0p[o0 + py];
            lu[2] = c0p[o1 + p00];
            lu[3] = c1p[o0 + p00];
            lu[4] = o0p[o0 + px];
            lu[5] = o0p[o0 + py];
            lu[6] = o0p[o1 + p00];
            lu[7] = o1p[o0 + p00];
#pragma unroll
            for (int i = 0; i < 4; ++i) lm[i] = mu[i * cs + qq];
        };
        load(0, q);
        for (int qt = 0; qt <= m; ++qt) {
            const float fcx = lu[0], fcy = lu[1], fct = lu[2], fcz = lu[3];
            const float fox = lu[4], foy = lu[5], fot = lu[6], foz = lu[7];
            float mv[4], ps[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) mv[i] = lm[i];
            if (qt < m) load(qt + 1, q + st);
            const float h[4] = {sg * (fcx - fc), sg * (fcy - fc), sgt * (fct - fc), sg * (fcz - fc)};
            const float ho[4] = {sg * (fox - fo), sg * (foy - fo), sgt * (fot - fo), sg * (foz - fo)};
            float za2 = 0.f;
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                ps[i] = h[i] + mv[i] * rinv;  // solve_reg_ker, admm.cu:49-52
                za2 += ps[i] * ps[i];
            }
            const float za = sqrtf(za2);
            const float shr = (za <= thr) ? 0.f : 1.0f - thr / za;  // shrink factor of the 4-vector
            float r2 = 0.f, s2 = 0.f;
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                ps[i] = ps[i] * shr;
                psi[i * cs + q] = ps[i];
                mu[i * cs + q] = mv[i] + rho * h[i] - rho * ps[i];  // lin4(mu,h2,psi,1,rho,-rho)
                const float dr = h[i] - ps[i], ds = ho[i] - h[i];
                r2 += dr * dr;
                s2 += ds * ds;
            }
            a0 += r2;
            a1 += s2;
            if (inner_xyz && qt >= 1) {  // voxel q-1 = (x0, y0, t0, z0) inside the chunk
                const float dd = fc - fo;
                a2 = fmaf(dd, dd, a2);
            }
            fc = fct;
            fo = fot;
            q += st;
        }
    }
    const long long bid = ((long long)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
    block_reduce3<8>((double)a0, (double)a1, (double)a2, partials + 3 * bid);
}

int shrink_blocks(const TvGeo &t, int nchunks) {
    return ((t.n + 1 + 31) / 32) * ((t.n + 1 + 7) / 8) * nchunks * (t.nzp + 1);
}

int launch_shrink(const float *u_cur, const float *u_old, float *psi, float *mu, const float *rho,
                  float lambda0, int c0, int nchunks_total, const TvGeo &t, double *partials,
                  cudaStream_t s) {
    dim3 bs(32, 8), gs((t.n + 1 + 31) / 32, (t.n + 1 + 7) / 8, t.nchunks * (t.nzp + 1));
    k_shrink<<<gs, bs, 0, s>>>(u_cur, u_old, psi, mu, rho, lambda0, t, c0, nchunks_total, partials);
    LAUNCH_CHECK("k_shrink");
    return (int)(gs.x * gs.y * gs.z);
}

// ---------------------------------------------------------------------------
// Fixed-order FP64 sum of the shrink partials and the rho rule
// (rectv.cu:223-232): r = sum |h-psi|^2, s = rho^2 sum |dG u|^2;
// r > 10 s -> rho *= 2, s > 10 r -> rho *= 0.5.
// stats row = (||u_new - u_old||^2, rho_new, r, s); *iter_ctr counts rows.
// ---------------------------------------------------------------------------
__global__ void k_reduce_rho(const double *__restrict__ partials, int nparts, float *rho,
                             double *stats, int *iter_ctr, int stats_cap) {
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
        const float r0 = *rho;
        const double r = sh[0][0];
        const double sv = (double)r0 * (double)r0 * sh[1][0];
        float rn = r0;
        if (r > 10.0 * sv) rn = r0 * 2.0f;
        else if (sv > 10.0 * r) rn = r0 * 0.5f;
        *rho = rn;
        const int it = *iter_ctr;
        if (it < stats_cap) {
            stats[4 * it + 0] = sh[2][0];
            stats[4 * it + 1] = rn;
            stats[4 * it + 2] = r;
            stats[4 * it + 3] = sv;
        }
        *iter_ctr = it + 1;
    }
}

// First stage: block b sums its contiguous share of the partials, in order.
__global__ void k_sum_stage1(const double *__restrict__ partials, int nparts, double *__restrict__ out) {
    __shared__ double sh[3][256];
    const int per = (nparts + gridDim.x - 1) / gridDim.x;
    const int lo = blockIdx.x * per, hi = min(nparts, lo + per);
    double a = 0, b = 0, c = 0;
    for (int i = lo + threadIdx.x; i < hi; i += blockDim.x) {
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
        out[3 * blockIdx.x] = sh[0][0];
        out[3 * blockIdx.x + 1] = sh[1][0];
        out[3 * blockIdx.x + 2] = sh[2][0];
    }
}

int reduce_stage1_parts() { return 256; }

void launch_reduce_rho(const double *partials, int nparts, double *stage1, float *rho, double *stats, int *ctr,
                       int cap, cudaStream_t s) {
    k_sum_stage1<<<256, 256, 0, s>>>(partials, nparts, stage1);
    LAUNCH_CHECK("k_sum_stage1");
    k_reduce_rho<<<1, 256, 0, s>>>(stage1, 256, rho, stats, ctr, cap);
    LAUNCH_CHECK("k_reduce_rho");
}

// ---------------------------------------------------------------------------
// Reference-layout gradient (extendf + gradf, kernels_operators.cuh:4-44):
// fm [nzp+2][m][n][n] with halo slabs at 0 and nzp+1, h2 float4
// [nzp+1][m+1][n+1][n+1].
// ---------------------------------------------------------------------------
__global__ void k_gradient_ref(const float *__restrict__ fm, int zbase, float4 *__restrict__ h2, int flgl,
                               int flgr, TvGeo t) {
    const int qx = blockIdx.x * blockDim.x + threadIdx.x;
    const int qy = blockIdx.y * blockDim.y + threadIdx.y;
    const int pl = blockIdx.z;
    const int n = t.n, m = t.m, nzp = t.nzp;
    const int qt = pl % (m + 1), qz = pl / (m + 1);
    if (qx > n || qy > n) return;
    auto fe = [&](int a, int b, int c, int d) -> float {
        const int x = clampi(a - 1, 0, n - 1), y = clampi(b - 1, 0, n - 1), tt = clampi(c - 1, 0, m - 1);
        const int z = clampi(d - 1, -flgl, nzp - 1 + flgr) + zbase;
        return fm[(((long long)z * m + tt) * n + y) * n + x];
    };
    const float f0 = fe(qx, qy, qt, qz);
    const float s = t.sg;
    float4 h;
    h.x = (fe(qx + 1, qy, qt, qz) - f0) * s;
    h.y = (fe(qx, qy + 1, qt, qz) - f0) * s;
    h.z = (fe(qx, qy, qt + 1, qz) - f0) * s * t.lambda1;
    h.w = (fe(qx, qy, qt, qz + 1) - f0) * s;
    h2[(((long long)qz * (m + 1) + qt) * (n + 1) + qy) * (n + 1) + qx] = h;
}

void launch_gradient_ref(const float *fm, int zbase, float *h2, int flgl, int flgr, const TvGeo &t,
                         cudaStream_t s) {
    dim3 bs(32, 8), gs((t.n + 1 + 31) / 32, (t.n + 1 + 7) / 8, (t.nzp + 1) * (t.m + 1));
    k_gradient_ref<<<gs, bs, 0, s>>>(fm, zbase, reinterpret_cast<float4 *>(h2), flgl, flgr, t);
    LAUNCH_CHECK("k_gradient_ref");
}

// Reference-layout divergence (div, kernels_operators.cuh:46-73): four
// separately rounded accumulations, as in the reference.
__global__ void k_divergent_ref(float *__restrict__ fn, const float4 *__restrict__ h2, float tau,
                                TvGeo t) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int pl = blockIdx.z;
    const int n = t.n, m = t.m;
    const int tt = pl % m, z = pl / m;
    if (x >= n || y >= n) return;
    const long long v = (((long long)z * m + tt) * n + y) * n + x;
    const long long sy = n + 1, st = sy * (n + 1), sz = st * (m + 1);
    const long long q = (z + 1) * sz + (tt + 1) * st + (y + 1) * sy + (x + 1);
    const float s = t.sd;
    float f = fn[v];
    f += tau * (h2[q - 1].x - h2[q].x) * s;
    f += tau * (h2[q - sy].y - h2[q].y) * s;
    f += tau * (h2[q - st].z - h2[q].z) * s * t.lambda1;
    f += tau * (h2[q - sz].w - h2[q].w) * s;
    fn[v] = f;
}

void launch_divergent_ref(float *fn, const float *h2, float tau, const TvGeo &t, cudaStream_t s) {
    dim3 bs(32, 8), gs((t.n + 31) / 32, (t.n + 7) / 8, t.nzp * t.m);
    k_divergent_ref<<<gs, bs, 0, s>>>(fn, reinterpret_cast<const float4 *>(h2), tau, t);
    LAUNCH_CHECK("k_divergent_ref");
}

// ---------------------------------------------------------------------------
// FP64 dot product sum_i a_i b_i of float32 arrays, two fixed-order passes.
// ---------------------------------------------------------------------------
constexpr int kDotParts = 1024;
int dot_parts() { return kDotParts; }

__global__ void k_dot_part(const float *__restrict__ a, const float *__restrict__ b, long long count,
                           double *__restrict__ partials) {
    double acc = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count;
         i += (long long)gridDim.x * blockDim.x)
        acc += (double)a[i] * (double)b[i];
    __shared__ double sh[256];
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) partials[blockIdx.x] = sh[0];
}

__global__ void k_dot_final(const double *__restrict__ partials, int nparts, double *out) {
    __shared__ double sh[256];
    double acc = 0.0;
    for (int i = threadIdx.x; i < nparts; i += blockDim.x) acc += partials[i];
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out += sh[0];
}

void launch_dot(const float *a, const float *b, long long count, double *partials, int nparts,
                double *out, cudaStream_t s) {
    k_dot_part<<<nparts, 256, 0, s>>>(a, b, count, partials);
    LAUNCH_CHECK("k_dot_part");
    k_dot_final<<<1, 256, 0, s>>>(partials, nparts, out);
    LAUNCH_CHECK("k_dot_final");
}

}  // namespace rectv
