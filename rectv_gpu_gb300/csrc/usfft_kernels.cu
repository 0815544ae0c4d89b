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
#include "usfft_common.cuh"

namespace rectv {

namespace {

__device__ __forceinline__ void cp_async8(void *smem, const void *gmem) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(gmem) : "memory");
}

__device__ __forceinline__ void cp_async_wait_all() {
    asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
}

}  // namespace

// ---------------------------------------------------------------------------
// Forward: deapodise, zero-pad to P x P and modulate by (-1)^(X+Y)
// (divphi + fftshift, kernels_radonusfft.cuh:4-38), writing the real input of
// the in-place R2C transform: row Y of image img starts at complex element
// img_fwd*img + qoff + Y*qp (2*qp floats per row; the P reals are written).
// One block per row, 16-byte stores; rows outside the image are zeros.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256)
    k_deapod_pad(const float *__restrict__ u, float2 *__restrict__ spec, const float *__restrict__ dp, UsGeo g,
                 float inv4n2) {
    const int Y = blockIdx.x;
    const long long img = blockIdx.y;
    const int n = g.n;
    float2 *row = spec + img * g.img_fwd + g.qoff + (long long)Y * g.qp;  // 16-byte aligned (qp, qoff even)
    float4 *row4 = reinterpret_cast<float4 *>(row);
    const int n4 = n / 2;  // float4 stores: reals 4i .. 4i+3
    const int y = Y - n / 2;
    if (y < 0 || y >= n) {
        for (int i = threadIdx.x; i < n4; i += blockDim.x) row4[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        if ((n & 1) && threadIdx.x == 0) row[n - 1] = make_float2(0.f, 0.f);
        return;
    }
    const float *ur = u + (img * n + y) * (long long)n;
    const float sy = ((Y & 1) ? -dp[y] : dp[y]) * inv4n2;
    auto val = [&](int X) {  // real X of the padded row; (-1)^X of the fftshift
        const int x = X - n / 2;
        if (x < 0 || x >= n) return 0.f;
        const float v = __ldg(ur + x) * __ldg(dp + x) * sy;
        return (X & 1) ? -v : v;
    };
    for (int i = threadIdx.x; i < n4; i += blockDim.x) {
        const int X = 4 * i;
        row4[i] = make_float4(val(X), val(X + 1), val(X + 2), val(X + 3));
    }
    if ((n & 1) && threadIdx.x == 0) row[n - 1] = make_float2(val(2 * n - 2), val(2 * n - 1));
}

void launch_deapod_pad(const float *u, float *spec, int nimg, const float *deapod, const UsGeo &g,
                       cudaStream_t s) {
    dim3 gs(g.P, nimg);
    const float inv4n2 = (float)(1.0 / (4.0 * g.n * (double)g.n));
    k_deapod_pad<<<gs, 256, 0, s>>>(u, reinterpret_cast<float2 *>(spec), deapod, g, inv4n2);
    LAUNCH_CHECK("k_deapod_pad");
}

// ---------------------------------------------------------------------------
// Halo of the stored forward spectra: cell (y, x) of the window rows
// [-kHalo, P+kHalo) x columns [-kHalo, n+kHalo) outside the R2C output gets
// the periodic full-spectrum value F(y mod P, x mod P), read through the
// Hermitian symmetry F(a, b) = conj F(-a, -b) of a real input when b > n.
// One thread per halo cell: 2 kHalo full rows, then 2 kHalo - 1 columns of
// every interior row.
// ---------------------------------------------------------------------------
__global__ void k_spec_halo(float2 *__restrict__ spec, UsGeo g) {
    const int P = g.P, n = g.n;
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long wide = (long long)(2 * kHalo) * g.qp;  // cells of the full halo rows
    const int side = g.qp - (n + 1);                        // halo columns of an interior row
    if (e >= wide + (long long)P * side) return;
    int y, x;
    if (e < wide) {
        const int r = (int)(e / g.qp);
        x = (int)(e - (long long)r * g.qp) - kHalo;
        y = (r < kHalo) ? r - kHalo : P + (r - kHalo);
    } else {
        const long long e2 = e - wide;
        y = (int)(e2 / side);
        const int c = (int)(e2 - (long long)y * side);
        x = (c < kHalo) ? c - kHalo : n + 1 + (c - kHalo);
    }
    float2 *img = spec + (long long)blockIdx.y * g.img_fwd + g.qoff;
    const int a = ((y % P) + P) % P, b = ((x % P) + P) % P;
    float2 v;
    if (b <= n) {
        v = img[(long long)a * g.qp + b];
    } else {
        v = img[(long long)((P - a) % P) * g.qp + (P - b)];
        v.y = -v.y;
    }
    img[(long long)y * g.qp + x] = v;
}

void launch_spec_halo(float2 *spec, int nimg, const UsGeo &g, cudaStream_t s) {
    const long long cells = (long long)(2 * kHalo) * g.qp + (long long)g.P * (g.qp - (g.n + 1));
    dim3 gs((unsigned)((cells + 255) / 256), nimg);
    k_spec_halo<<<gs, 256, 0, s>>>(spec, g);
    LAUNCH_CHECK("k_spec_halo");
}

// ---------------------------------------------------------------------------
// Per-sample table built once per block in shared memory, one thread per
// sample: the 9+9 separable Gaussian weights, the stencil position in the
// block's tile, the angle/detector indices and a complex factor.
// ---------------------------------------------------------------------------
constexpr int kCH = 256;  // samples per table
constexpr int kThreads = 512;  // threads per gather/scatter block
constexpr int kWS = 28;   // floats per weight row: ex[9], ey[9], ex_im[9], 1 pad (16-byte rows)

struct EntryTab {
    float w[kCH][kWS];
    int cb[kCH];   // gather: float2 offset of the stencil origin in the tile (-1: invalid)
                   // scatter: packed (dx + 32) | (dy + 32) << 8
    int th[kCH];
    int k[kCH];
    float2 f[kCH];  // gather: (pi/mu)/n (-1)^(k+1) shiftfwd(k); scatter: E(theta, k) of this slice
};


// Scatter block's shared memory: sample table, per-ray grids of one batch of
// rays, and the ray index of each table row.
constexpr int kSegBatch = 16;

template <int T>
struct ScatterSmem {
    EntryTab tab;
    float v[kSegBatch][2][T * T];  // per-ray grids, real and imaginary planes
    float4 kr[kSegBatch][8];       // per-ray mixing rows K'(theta, jbase + j), j < 16
    int seg_of[kCH];     // ray (segment) index of each table row
    int seg_first[kCH];  // first table row of each segment
    int wsum[8];
};

// ---------------------------------------------------------------------------
// Forward gather (gather TOMO_FWD, kernels_radonusfft.cuh:81-144, fused with
// the basis sum of operators.cu:143-152 and shift/fftshift of
// radonusfft.cu:96-97).  One block per (work item, slice); a work item is a
// 16x16 tile of the spectrum and up to kCH samples whose stencil origin lies
// in it.  The block stages the (16+8)^2 cells x MP time samples of its tile,
// builds the sample table, then each group of MP lanes computes one sample:
// lane j reads time sample j's complex value per tap (64-bit loads, a
// 128-byte row per sample), and the group sums K'(theta, j) H_j with
// shuffles.  jbase selects a group of MP time samples (m > 16 runs several
// passes, accumulating into rows).
// ---------------------------------------------------------------------------
template <int MP, int T>
__global__ void __launch_bounds__(kThreads)
    k_gather_fwd(const float2 *__restrict__ spec, float2 *__restrict__ rows,
                 const uint32_t *__restrict__ pts, const int4 *__restrict__ items,
                 const float2 *__restrict__ sincos, const float2 *__restrict__ kmat,
                 const float2 *__restrict__ shiftf, UsGeo g, int jbase, int accumulate,
                 int *__restrict__ err) {
    constexpr int TW = T + 2 * kR;
    constexpr int EPW = 32 / MP;  // samples per warp
    extern __shared__ float4 smraw[];
    float2 *tile = reinterpret_cast<float2 *>(smraw);  // [TW*TW][MP]
    EntryTab &tab = *reinterpret_cast<EntryTab *>(tile + TW * TW * MP);
    const int4 it = items[blockIdx.x];
    const int z = blockIdx.y;
    const int tyi = it.x / g.NT, txi = it.x - tyi * g.NT;
    const int P = g.P, half = P / 2;
    const int count = it.z;
    const float2 *img0 = spec + (long long)z * g.m * g.img_fwd;

    // ---- stage the tile with asynchronous copies, one time-sample plane at
    // a time with consecutive threads on consecutive cells (coalesced reads).
    // Cell c, time sample j sits at float2 c*MP + (j ^ (column & (MP-1))): the
    // XOR swizzle keeps both these stores and the compute loop's 128-byte rows
    // free of bank conflicts.  The post-FFT fftshift sign (-1)^(X+Y) of a cell
    // is (-1)^(column+row) of its tile position, and cells right of the
    // Nyquist column are read through the Hermitian symmetry of the real-input
    // FFT (conjugated); both signs are folded into the tap weights. ----
    {
        constexpr int NC = TW * TW;
        for (int cell = threadIdx.x; cell < NC; cell += blockDim.x) {
            const int row = cell / TW, col = cell - row * TW;
            int KY = tyi * T - kR + row;
            KY += (KY < 0) ? P : 0;
            KY -= (KY >= P) ? P : 0;
            int KX = txi * T - kR + col;
            KX += (KX < 0) ? P : 0;
            KX -= (KX >= P) ? P : 0;
            const long long so = g.qoff + ((KX <= half) ? (long long)KY * g.qp + KX
                                                        : (long long)(KY ? P - KY : 0) * g.qp + (P - KX));
            const float2 *src = img0 + (long long)jbase * g.img_fwd + so;
            float2 *dst = tile + cell * MP;
            const int sw = col & (MP - 1);
#pragma unroll 4
            for (int j = 0; j < MP; ++j) {
                if (jbase + j < g.m) cp_async8(dst + (j ^ sw), src + (long long)j * g.img_fwd);
                else dst[j ^ sw] = make_float2(0.f, 0.f);
            }
        }
        cp_async_wait_all();
    }
    // ---- sample table ----
    for (int e = threadIdx.x; e < count; e += blockDim.x) {
        const uint32_t id = __ldg(pts + it.y + e);
        const int th = id / (uint32_t)g.n;
        const int k = id - th * g.n;
        float x0, y0;
        int fx, fy;
        sample_pos(k, __ldg(sincos + th), g, x0, y0, fx, fy);
        const int lx0 = g.n + fx - txi * T;
        const int ly0 = g.n + fy - tyi * T;
        float ex[kTaps], ey[kTaps];
        tap_weights(fx, x0, g, ex);
        tap_weights(fy, y0, g, ey);
#pragma unroll
        for (int i = 0; i < kTaps; ++i) {  // (-1)^(a+b) of the fftshift sign
            const float sx = (i & 1) ? -ex[i] : ex[i];
            int KX = txi * T - kR + lx0 + i;  // conjugated columns flip the imaginary weight
            KX += (KX < 0) ? P : 0;
            KX -= (KX >= P) ? P : 0;
            tab.w[e][i] = sx;
            tab.w[e][kTaps + i] = (i & 1) ? -ey[i] : ey[i];
            tab.w[e][2 * kTaps + i] = (KX > half) ? -sx : sx;
        }
        if (lx0 < 0 || lx0 >= T || ly0 < 0 || ly0 >= T) {  // host/device bin disagreement
            atomicAdd(err, 1);
            tab.cb[e] = -1;
        } else {
            tab.cb[e] = ((ly0 * TW + lx0) * MP) | (lx0 << 20);
        }
        tab.th[e] = th;
        tab.k[e] = k;
        float2 sh = __ldg(shiftf + k);
        float c = (k & 1) ? g.cw : -g.cw;  // (-1)^(k+1) and (pi/mu)/n
        if ((lx0 + ly0) & 1) c = -c;        // fftshift sign of the stencil origin
        tab.f[e] = make_float2(sh.x * c, sh.y * c);
    }
    __syncthreads();

    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int grp = lane / MP, j = lane - grp * MP;
    const int jg = jbase + j;
    const unsigned full = 0xffffffffu;
    for (int e0 = wid * EPW; e0 < count; e0 += nw * EPW) {
        const int e = e0 + grp;
        bool valid = e < count;
        const int ee = valid ? e : e0;
        int cb = tab.cb[ee];
        int lx0 = cb >> 20;
        cb &= (1 << 20) - 1;
        if (tab.cb[ee] < 0) {
            valid = false;
            cb = 0;
            lx0 = 0;
        }
        float w[kWS];
        {
            const float4 *wr = reinterpret_cast<const float4 *>(tab.w[ee]);
#pragma unroll
            for (int i = 0; i < kWS / 4; ++i) {
                const float4 v = wr[i];
                w[4 * i] = v.x;
                w[4 * i + 1] = v.y;
                w[4 * i + 2] = v.z;
                w[4 * i + 3] = v.w;
            }
        }
        const int th = tab.th[ee];
        const float2 kv = (jg < g.m) ? __ldg(kmat + (long long)th * g.m + jg) : make_float2(0.f, 0.f);
        const float2 *bcol[kTaps];  // per tap column: swizzled slot of time sample j
#pragma unroll
        for (int b = 0; b < kTaps; ++b) bcol[b] = tile + cb + b * MP + (j ^ ((lx0 + b) & (MP - 1)));
        float ax = 0.f, ay = 0.f;
#pragma unroll
        for (int a = 0; a < kTaps; ++a) {
            float rx = 0.f, ry = 0.f;
#pragma unroll
            for (int b = 0; b < kTaps; ++b) {
                const float2 v = bcol[b][a * TW * MP];
                rx = fmaf(w[b], v.x, rx);
                ry = fmaf(w[2 * kTaps + b], v.y, ry);
            }
            ax = fmaf(w[kTaps + a], rx, ax);
            ay = fmaf(w[kTaps + a], ry, ay);
        }
        // time-sample mixing: sum_j K'(theta, j) H_j over the group's lanes
        float px = ax * kv.x - ay * kv.y;
        float py = ax * kv.y + ay * kv.x;
#pragma unroll
        for (int o = 1; o < MP; o <<= 1) {
            px += __shfl_xor_sync(full, px, o);
            py += __shfl_xor_sync(full, py, o);
        }
        if (valid && j == 0) {
            float2 r = cmul(make_float2(px, py), tab.f[ee]);
            float2 *dst = rows + ((long long)z * g.ntheta + th) * g.n + tab.k[ee];
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
    return (size_t)(g.T + 2 * kR) * (g.T + 2 * kR) * mp_for(g.m) * sizeof(float2) + sizeof(EntryTab);
}
size_t scatter_adj_smem(const UsGeo &g) { return sizeof(ScatterSmem<16>); }
int table_capacity() { return kCH; }

template <int MP, int T>
static void gather_fwd_t(const float2 *spec, float2 *rows, int zb, const GeoDev &gd, const UsGeo &g,
                         int jbase, int accumulate, int *err, cudaStream_t s) {
    const size_t smem = (size_t)(T + 2 * kR) * (T + 2 * kR) * MP * sizeof(float2) + sizeof(EntryTab);
    dim3 gs(gd.n_fwd_items, zb);
    k_gather_fwd<MP, T><<<gs, kThreads, smem, s>>>(spec, rows, gd.fwd_pts, gd.fwd_items, gd.sincos, gd.kmat,
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
                       const CUtensorMap *tmap, cudaStream_t s) {
    const long long nrows = (long long)zb * g.ntheta;
    k_zero_k0<<<(unsigned)((nrows + 255) / 256), 256, 0, s>>>(rows, nrows, g.n);
    LAUNCH_CHECK("k_zero_k0");
    if (g.T != 16) throw Error(1, "tile size must be 16");
    if (gd.dirs) {  // rays grouped by direction: one interpolation per position (dir_kernels.cu)
        for (int jb = 0; jb < g.m; jb += 16) launch_gather_dir(rows, spec, zb, gd, g, jb, jb > 0, s);
        return;
    }
    const int mp = mp_for(g.m);
    for (int jb = 0; jb < g.m; jb += 16) {
        const int acc = jb > 0;
        // the plan gives items with several samples per ray to the tensor-core
        // gather from 8 time samples up (any group size: missing samples are zero)
        if (gd.n_fwd_tc_items > 0) launch_gather_tc(rows, zb, gd, g, *tmap, jb, acc, s);
        if (gd.n_fwd_items == 0) continue;
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
// weights of operators.cu:171-176 and the pre-IFFT fftshift).
//
// One block per (16x16 tile of the periodic grid, slice).  The samples whose
// stencil touches the tile arrive sorted by angle.  Along one ray theta the
// time-sample weights conj(K'(theta, j)) are the same for every sample, so the
// block works per ray ("segment"), in batches of kSegBatch rays:
//  1. a warp per sample, lanes on its 81 taps, adds w E(theta, k) into the
//     ray's single-complex grid V_ray (shared memory);
//  2. thread = cell adds conj(K'(theta, j)) V_ray(cell) to the cell's MP
//     complex time-sample accumulators, held in registers.
// The tile is stored once at the end (added, for a tile split over blocks).
// ---------------------------------------------------------------------------
template <int MP, int T>
__global__ void __launch_bounds__(T * T, 3)
    k_scatter_adj(const float2 *__restrict__ rowsc, float2 *__restrict__ spec,
                  const uint32_t *__restrict__ pts, const int4 *__restrict__ items,
                  const float2 *__restrict__ sincos, const float2 *__restrict__ kmat,
                  const float2 *__restrict__ shifta, UsGeo g, int jbase) {
    static_assert(T == 16, "one thread per cell of a 16x16 tile");
    extern __shared__ float4 smraw[];
    ScatterSmem<T> &sm = *reinterpret_cast<ScatterSmem<T> *>(smraw);
    EntryTab &tab = sm.tab;
    const int4 it = items[blockIdx.x];
    const int z = blockIdx.y;
    const int tyi = it.x / g.NT, txi = it.x - tyi * g.NT;
    const int P = g.P, half = P / 2, hn = g.n / 2 + 1;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    constexpr int NW = T * T / 32;
    const float2 *rz = rowsc + (long long)z * g.ntheta * hn;
    // this lane's taps t = lane, lane+32, lane+64 (< 81): row a = t/9, column b = t%9
    int ta[3], tb[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const int t = lane + 32 * i;
        ta[i] = (t < kTaps * kTaps) ? t / kTaps : 1000;
        tb[i] = t - (t / kTaps) * kTaps;
    }
    float ar[MP], ai[MP];
#pragma unroll
    for (int j = 0; j < MP; ++j) ar[j] = ai[j] = 0.f;
    for (int c0 = 0; c0 < it.z; c0 += kCH) {
        const int cnt = min(kCH, it.z - c0);
        __syncthreads();  // previous table consumed
        for (int e = tid; e < cnt; e += blockDim.x) {
            const uint32_t id = __ldg(pts + it.y + c0 + e);
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
            float ex[kTaps], ey[kTaps];
            tap_weights(fx, x0, g, ex);
            tap_weights(fy, y0, g, ey);
#pragma unroll
            for (int i = 0; i < kTaps; ++i) {
                tab.w[e][i] = ex[i];
                tab.w[e][kTaps + i] = ey[i];
            }
            // stencils of listed samples start within [-2r, T) of the tile
            tab.cb[e] = ((dx + 32) & 0xff) | (((dy + 32) & 0xff) << 8);
            tab.th[e] = th;
            // E = (-1)^(k+1) shiftadj(k) FFT(row)(k) (pi/mu)/n  (Hermitian row spectrum)
            float2 R = (k <= g.n / 2) ? __ldg(rz + (long long)th * hn + k)
                                      : __ldg(rz + (long long)th * hn + (g.n - k));
            if (k > g.n / 2) R.y = -R.y;
            const float2 E = cmul(R, __ldg(shifta + k));
            const float c = (k & 1) ? g.cw : -g.cw;
            tab.f[e] = make_float2(E.x * c, E.y * c);
        }
        __syncthreads();
        // ---- segment index of each row: block-wide inclusive scan of ray starts ----
        int flag = 0;
        if (tid < cnt) flag = (tid == 0 || tab.th[tid] != tab.th[tid - 1]) ? 1 : 0;
        int incl = flag;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        if (lane == 31) sm.wsum[wid] = incl;
        __syncthreads();
        int base = 0, nseg = 0;
#pragma unroll
        for (int w = 0; w < NW; ++w) {
            const int v = sm.wsum[w];
            base += (w < wid) ? v : 0;
            nseg += v;
        }
        incl += base;
        if (tid < cnt) {
            sm.seg_of[tid] = incl - 1;
            if (flag) sm.seg_first[incl - 1] = tid;
        }
        for (int sb = 0; sb < nseg; sb += kSegBatch) {
            const int nb = min(kSegBatch, nseg - sb);
            __syncthreads();  // seg tables written; previous batch mixed
            for (int s = 0; s < nb; ++s) {
                sm.v[s][0][tid] = 0.f;
                sm.v[s][1][tid] = 0.f;
            }
            if (tid < nb * 16) {  // stage the batch's mixing rows (zero beyond m)
                const int s = tid >> 4, j = tid & 15;
                const int th = tab.th[sm.seg_first[sb + s]];
                const float2 kv =
                    (jbase + j < g.m) ? __ldg(kmat + (long long)th * g.m + jbase + j) : make_float2(0.f, 0.f);
                reinterpret_cast<float2 *>(sm.kr[s])[j] = kv;
            }
            __syncthreads();
            // ---- 1. rays' grids: a warp per ray (its samples in order, so the
            // sums are reproducible), lanes on the taps of one sample ----
            for (int s = wid; s < nb; s += NW)
            for (int e = sm.seg_first[sb + s], e_end = (sb + s + 1 < nseg) ? sm.seg_first[sb + s + 1] : cnt;
                 e < e_end; ++e) {
                const int pk = tab.cb[e];
                const int dx = (pk & 0xff) - 32, dy = ((pk >> 8) & 0xff) - 32;
                const float2 E = tab.f[e];
                float *vs = sm.v[s][0];
#pragma unroll
                for (int i = 0; i < 3; ++i) {
                    const int cy = dy + ta[i], cx = dx + tb[i];
                    if ((unsigned)cy < (unsigned)T && (unsigned)cx < (unsigned)T) {
                        const float w = tab.w[e][tb[i]] * tab.w[e][kTaps + ta[i]];
                        const unsigned sa = (unsigned)__cvta_generic_to_shared(vs + cy * T + cx);
                        asm volatile("red.shared.add.f32 [%0], %1;\n" ::"r"(sa), "f"(w * E.x) : "memory");
                        asm volatile("red.shared.add.f32 [%0+1024], %1;\n" ::"r"(sa), "f"(w * E.y) : "memory");
                    }
                }
            }
            __syncthreads();
            // ---- 2. thread = cell: acc_j += conj(K'(theta, j)) V_ray(cell) ----
            for (int s = 0; s < nb; ++s) {
                const float2 v = make_float2(sm.v[s][0][tid], sm.v[s][1][tid]);
                if (v.x != 0.f || v.y != 0.f) {
#pragma unroll
                    for (int jj = 0; jj < (MP + 1) / 2; ++jj) {
                        const float4 kv = sm.kr[s][jj];
                        ar[2 * jj] = fmaf(kv.x, v.x, fmaf(kv.y, v.y, ar[2 * jj]));
                        ai[2 * jj] = fmaf(kv.x, v.y, fmaf(-kv.y, v.x, ai[2 * jj]));
                        if (2 * jj + 1 < MP) {
                            ar[2 * jj + 1] = fmaf(kv.z, v.x, fmaf(kv.w, v.y, ar[2 * jj + 1]));
                            ai[2 * jj + 1] = fmaf(kv.z, v.y, fmaf(-kv.w, v.x, ai[2 * jj + 1]));
                        }
                    }
                }
            }
        }
    }
    // ---- store the cell (pre-IFFT fftshift sign); split tiles add ----
    const int ly = tid / T, lx = tid - (tid / T) * T;
    const int KY = tyi * T + ly, KX = txi * T + lx;
    if (KY < P && KX < P) {
        const float sg = ((KX + KY) & 1) ? -1.f : 1.f;
        float2 *dst = spec + ((long long)z * g.m + jbase) * g.img_adj + (long long)KY * P + KX;
#pragma unroll
        for (int j = 0; j < MP; ++j) {
            if (jbase + j >= g.m) break;
            const float2 v = make_float2(sg * ar[j], sg * ai[j]);
            float2 *d = dst + (long long)j * g.img_adj;
            if (it.w) {
                atomicAdd(&d->x, v.x);
                atomicAdd(&d->y, v.y);
            } else {
                *d = v;
            }
        }
    }
}

template <int MP, int T>
static void scatter_adj_t(const float2 *rowsc, float2 *spec, int zb, const GeoDev &gd,
                          const UsGeo &g, int jbase, cudaStream_t s) {
    const size_t smem = sizeof(ScatterSmem<T>);
    dim3 gs(gd.n_adj_items, zb);
    k_scatter_adj<MP, T><<<gs, T * T, smem, s>>>(rowsc, spec, gd.adj_pts, gd.adj_items, gd.sincos, gd.kmat,
                                               gd.shiftadj, g, jbase);
    LAUNCH_CHECK("k_scatter_adj");
}

void launch_scatter_adj(const float2 *rowsc, float2 *spec, int zb, const GeoDev &gd,
                        const UsGeo &g, cudaStream_t s) {
    if (g.T != 16) throw Error(1, "tile size must be 16");
    if (gd.dirs) {  // rays grouped by direction, into the Hermitian half planes (dir_kernels.cu)
        for (int jb = 0; jb < g.m; jb += 16) launch_scatter_dir(rowsc, spec, zb, gd, g, jb, s);
        return;
    }
    const int mp = mp_for(g.m);
    for (int jb = 0; jb < g.m; jb += 16) {
        // the tensor-core scatter fills the Hermitian half planes the spectra
        // buffer is sized for (from 8 time samples up)
        if (gd.tc_scatter) {
            launch_scatter_tc(rowsc, spec, zb, gd, g, jb, s);
            continue;
        }
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

// Same epilogue after the C2R inverse of the Hermitian half planes: real
// images with rows of 2 (P/2+1) floats.
__global__ void k_crop_accum_real(const float *__restrict__ out, float *__restrict__ u,
                                  const float *__restrict__ dp, int n, int P, long long img_real, float c) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    const long long img = blockIdx.z;
    if (x >= n) return;
    const int X = x + n / 2, Y = y + n / 2;
    float v = out[img * img_real + (long long)Y * (P + 2) + X];
    v = ((X + Y) & 1) ? -v : v;
    u[(img * n + y) * n + x] += c * v * dp[x] * dp[y];
}

void launch_crop_accum_real(const float *out, float *u, int zb, float tau, const float *deapod, const UsGeo &g,
                            cudaStream_t s) {
    dim3 gs((g.n + 255) / 256, g.n, zb * g.m);
    const double scale = 1.0 / std::sqrt((double)g.n * (double)g.ntheta);
    const float c = (float)(tau * scale / (4.0 * g.n * (double)g.n));
    const long long img_real = 2LL * g.P * (g.P / 2 + 1);
    k_crop_accum_real<<<gs, 256, 0, s>>>(out, u, deapod, g.n, g.P, img_real, c);
    LAUNCH_CHECK("k_crop_accum_real");
}

template <int MP, int T>
static void set_attrs() {
    const int fs = (int)((T + 2 * kR) * (T + 2 * kR) * MP * sizeof(float2) + sizeof(EntryTab));
    const int as = (int)sizeof(ScatterSmem<T>);
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
