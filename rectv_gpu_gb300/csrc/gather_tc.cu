// Forward USFFT gather on the tensor cores (tcgen05) with TMA staging, for
// work items whose samples lie on few rays (several samples per ray and tile:
// all but a handful of items at the centre of the spectrum).
//
// The forward operator needs, per polar sample p on ray theta,
//     sum_j K'(theta, j) sum_taps w(p, c) F_j(c)
// (gather, kernels_radonusfft.cuh:81-144, fused with the basis sum of
// operators.cu:143-152).  The sum over time samples j does not depend on the
// sample, only on its ray, so it is done first, for every cell c of the tile
// footprint and every ray crossing the tile:
//     G(c, theta) = sum_j F_j(c) K'(theta, j)                 (complex GEMM)
// after which each sample interpolates one complex value per tap from
// G(., theta) instead of m.  G is a [cells x 16] x [16 x rays] complex
// product, computed as a real [640 x 32] x [32 x 32] product per chunk of 16
// rays (K index 2j + re/im; N index 2r + re/im of G) with three TF32
// tensor-core terms for FP32 accuracy:
//     F K ~ Fhi Khi + Fhi Klo + Flo Khi
// where hi is the TF32 part (the tensor core truncates FP32 input to TF32)
// and lo = x - trunc(x), itself truncated to TF32 (relative error < 2^-20).
//
// One block (512 threads, one per SM) per (work item, 64 slices):
//  * once: the sample table (stencil origin, separable Gaussian weights with
//    the fftshift signs, row factor) and the item's rays; the B operands
//    (K' rows) when the item has at most two chunks of rays;
//  * per slice: one TMA box load brings the 24x24-cell footprint of the
//    16x16 floor tile, 16 time samples, from the halo-padded spectra into
//    shared memory (the next slice's box is loaded while this slice is
//    computed); threads convert it (Hermitian-mirrored tiles read the mirrored
//    box, conjugated) into the A operand in tensor memory, hi and lo parts;
//  * per chunk of 16 rays: 60 MMAs into the accumulator, issued by five
//    threads (one per M tile of 128 cells: its own accumulation chain);
//    the block moves G to shared memory, the next chunk's MMAs are issued,
//    and four threads per sample sum its 81 taps of G and write the row value
//    (times (-1)^(k+1) shift(k) (pi/mu)/n).
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include "rectv_internal.cuh"
#include "tcgen05.cuh"
#include "usfft_common.cuh"

namespace rectv {

namespace {

constexpr int kT = 16;                       // floor tile side
constexpr int kFW = kT + 2 * kR;             // footprint side (24)
constexpr int kBoxW = kFW + 2;               // box width: even start column of a mirrored footprint
constexpr int kCells = kFW * kFW;            // 576
constexpr int kGP = kFW + 1;                 // row pitch of G in shared memory (25: the four threads
                                             // of a sample read rows 8 B x 25 apart, on distinct banks)
constexpr int kMT = (kCells + 127) / 128;    // M tiles of 128 cells (5)
constexpr int kRays = 16;                    // rays per chunk
constexpr int kN = 2 * kRays;                // MMA N (32)
constexpr int kK = 32;                       // 16 time samples x (re, im)
constexpr int kTab = 256;                    // samples per work item
constexpr int kThr = 512;
constexpr int kWarps = kThr / 32;
constexpr int kZPer = 64;                    // slices per block at most (UsGeo::zper)
constexpr uint32_t kTmemCols = 512;
constexpr uint32_t kColAhi = 0;              // TMEM columns: A hi [mt*32, +32)
constexpr uint32_t kColAlo = kMT * kK;       //               A lo
constexpr uint32_t kColD = 2 * kMT * kK;     //               D    [mt*32, +32)
constexpr uint32_t kBoxBytes = 16 * kFW * kBoxW * 8;

// Core-matrix offset (floats) of element (row, kk) of a K-major FP32 operand
// with 32 K values per row (LBO 128 B, SBO 1024 B).
__device__ __forceinline__ int off32(int row, int kk) {
    return (row >> 3) * 256 + (kk >> 2) * 32 + (row & 7) * 4 + (kk & 3);
}

struct TcSmem {
    float2 box[16][kFW][kBoxW];          // TMA destination: 16 time samples x 24 rows x 26 cells
    float2 g[kRays][kFW * kGP];          // G of the current chunk's rays, cell (row, col) at row * kGP + col
    float bhi[2][kN * kK];               // B = K' rows, FP32 (double-buffered)
    float blo[2][kN * kK];               // B - trunc(B)
    float wx[kTab][12];                  // (-1)^b w_b of the 9 x taps
    float wy[kTab][12];                  // (-1)^a w_a of the 9 y taps
    int pos[kTab];                       // stencil origin cell in the footprint (-1: invalid)
    int th[kTab];
    int k[kTab];
    float2 f[kTab];                      // (-1)^(k+1) shiftfwd(k) (pi/mu)/n (-1)^(origin parity)
    int seg_of[kTab];
    int seg_first[kTab + 1];
    int wsum[kWarps];
    unsigned long long bar_mma, bar_tma;
    uint32_t tslot;
};

__device__ __forceinline__ void st32(uint32_t taddr, const float (&v)[32]) {
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};\n" ::"r"(
            taddr),
        "f"(v[0]), "f"(v[1]), "f"(v[2]), "f"(v[3]), "f"(v[4]), "f"(v[5]), "f"(v[6]), "f"(v[7]), "f"(v[8]), "f"(v[9]),
        "f"(v[10]), "f"(v[11]), "f"(v[12]), "f"(v[13]), "f"(v[14]), "f"(v[15])
        : "memory");
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};\n" ::"r"(
            taddr + 16),
        "f"(v[16]), "f"(v[17]), "f"(v[18]), "f"(v[19]), "f"(v[20]), "f"(v[21]), "f"(v[22]), "f"(v[23]), "f"(v[24]),
        "f"(v[25]), "f"(v[26]), "f"(v[27]), "f"(v[28]), "f"(v[29]), "f"(v[30]), "f"(v[31])
        : "memory");
}

// D (+)= A B^T, A [128 x 8] TF32 in tensor memory, B [N x 8] TF32 in shared memory.
__device__ __forceinline__ void mma_tf32_ts(uint32_t d, uint32_t a, uint64_t b, uint32_t id, uint32_t acc) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n}\n" ::"r"(d),
        "r"(a), "l"(b), "r"(id), "r"(acc)
        : "memory");
}

}  // namespace

__global__ void __launch_bounds__(kThr, 1)
    k_gather_tc(float2 *__restrict__ rows, const uint32_t *__restrict__ pts, const int4 *__restrict__ items,
                const float2 *__restrict__ sincos, const float2 *__restrict__ kmat,
                const float2 *__restrict__ shiftf, const __grid_constant__ CUtensorMap tmap, UsGeo g, int zb,
                int jbase, int accumulate, int *__restrict__ err) {
    extern __shared__ __align__(1024) unsigned char tc_smem_raw[];
    TcSmem &sm = *reinterpret_cast<TcSmem *>(tc_smem_raw);
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int4 it = items[blockIdx.x];
    const int zper = g.zper;
    const int z0 = blockIdx.y * zper, z1 = min(zb, z0 + zper);
    const int tyi = it.x / g.NT, txi = it.x - tyi * g.NT;
    const int P = g.P;
    const int cnt = min(it.z, kTab);
    // Footprint box in the halo-padded spectra (window origin (-kHalo, -kHalo)):
    // tiles left of the Nyquist column read the direct box, the others the
    // box of the mirrored cells (P - KY, P - KX), conjugated.
    const bool mirrored = txi * kT > g.n + 2;
    const int bx = mirrored ? 2 * (P - txi * kT - kR - kT + kHalo) : 2 * (txi * kT - kR + kHalo);
    const int by = mirrored ? P - tyi * kT - (kT + kR - 1) + kHalo : tyi * kT - kR + kHalo;

    if (wid == 0) tc::alloc(&sm.tslot, kTmemCols);
    if (tid == 0) {
        tc::mbar_init(&sm.bar_mma, kMT);  // one commit per M tile
        tc::mbar_init(&sm.bar_tma, 1);
        tc::fence_mbar_init();
    }
    auto tma_issue = [&](int z) {  // one thread: box of slice z, time samples [jbase, jbase + 16)
        const uint32_t bar = tc::smem_addr(&sm.bar_tma);
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"(kBoxBytes)
                     : "memory");
        asm volatile(
            "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, "
            "%4}], [%5];\n" ::"r"(tc::smem_addr(&sm.box[0][0][0])),
            "l"((unsigned long long)&tmap), "r"(bx), "r"(by), "r"(z * g.m + jbase), "r"(bar)
            : "memory");
    };
    __syncthreads();  // barriers initialised
    if (tid == 0) tma_issue(z0);

    // ---- sample table (the same for every slice) ----
    for (int e = tid; e < cnt; e += kThr) {
        const uint32_t id = __ldg(pts + it.y + e);
        const int th = id / (uint32_t)g.n;
        const int k = id - th * g.n;
        float x0, y0;
        int fx, fy;
        sample_pos(k, __ldg(sincos + th), g, x0, y0, fx, fy);
        const int lx0 = g.n + fx - txi * kT;
        const int ly0 = g.n + fy - tyi * kT;
        if (lx0 < 0 || lx0 >= kT || ly0 < 0 || ly0 >= kT) {  // host/device bin disagreement
            atomicAdd(err, 1);
            sm.pos[e] = -1;
        } else {
            sm.pos[e] = ly0 * kGP + lx0;
        }
        sm.th[e] = th;
        sm.k[e] = k;
#pragma unroll
        for (int b = 0; b < kTaps; ++b) {
            const float wxb = tap_weight(fx, b, x0, g), wyb = tap_weight(fy, b, y0, g);
            sm.wx[e][b] = (b & 1) ? -wxb : wxb;  // (-1)^b of the fftshift sign
            sm.wy[e][b] = (b & 1) ? -wyb : wyb;
        }
        const float2 sh = __ldg(shiftf + k);
        float cf = (k & 1) ? g.cw : -g.cw;  // (-1)^(k+1) and (pi/mu)/n
        if ((lx0 + ly0) & 1) cf = -cf;      // fftshift sign of the stencil origin
        sm.f[e] = make_float2(sh.x * cf, sh.y * cf);
    }
    __syncthreads();
    // ---- rays of the item (segments of equal theta; samples are theta-major) ----
    int nseg;
    {
        int flag = 0;
        if (tid < cnt) flag = (tid == 0 || sm.th[tid] != sm.th[tid - 1]) ? 1 : 0;
        int incl = flag;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        if (lane == 31) sm.wsum[wid] = incl;
        __syncthreads();
        int base = 0;
        nseg = 0;
#pragma unroll
        for (int w = 0; w < kWarps; ++w) {
            const int v = sm.wsum[w];
            base += (w < wid) ? v : 0;
            nseg += v;
        }
        incl += base;
        if (tid < cnt) {
            sm.seg_of[tid] = incl - 1;
            if (flag) sm.seg_first[incl - 1] = tid;
        }
        if (tid == 0) sm.seg_first[nseg] = cnt;
    }
    __syncthreads();
    const int nch = (nseg + kRays - 1) / kRays;

    // B rows of chunk ch into buffer buf: row 2r gives Re G, row 2r+1 Im G of
    // ray r; K index 2j (Re F_j) and 2j+1 (Im F_j).  Threads 0..255 = (row, 4 K values).
    auto stage_b = [&](int ch, int buf) {
        if (tid >= kN * kK / 4) return;
        const int nrow = tid >> 3, q4 = tid & 7;
        const int r = nrow >> 1, o = nrow & 1;
        const int s = ch * kRays + r;
        float bv[4] = {0.f, 0.f, 0.f, 0.f};
        if (s < nseg) {
            const int th = sm.th[sm.seg_first[s]];
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                const int j = 2 * q4 + i;
                float2 kv = make_float2(0.f, 0.f);
                if (jbase + j < g.m) kv = __ldg(kmat + (long long)th * g.m + jbase + j);
                if (o == 0) {
                    bv[2 * i] = kv.x;
                    bv[2 * i + 1] = -kv.y;
                } else {
                    bv[2 * i] = kv.y;
                    bv[2 * i + 1] = kv.x;
                }
            }
        }
        const int o32 = off32(nrow, 4 * q4);
        *reinterpret_cast<float4 *>(sm.bhi[buf] + o32) = make_float4(bv[0], bv[1], bv[2], bv[3]);
        *reinterpret_cast<float4 *>(sm.blo[buf] + o32) =
            make_float4(bv[0] - tc::trunc_tf32(bv[0]), bv[1] - tc::trunc_tf32(bv[1]),
                        bv[2] - tc::trunc_tf32(bv[2]), bv[3] - tc::trunc_tf32(bv[3]));
    };

    // G = A B^T for chunk ch (B in buffer buf), M tile mt, into the
    // accumulator; N = 16 when the chunk has at most 8 rays.
    auto issue = [&](uint32_t tbase, int ch, int buf, int mt) {
        const int nr = min(kRays, nseg - ch * kRays);
        const uint32_t IT = nr > 8 ? tc::idesc(tc::kFmtTF32, 128, 32) : tc::idesc(tc::kFmtTF32, 128, 16);
        const uint64_t dh = tc::sdesc(tc::smem_addr(sm.bhi[buf]), 128, 1024);
        const uint64_t dl = tc::sdesc(tc::smem_addr(sm.blo[buf]), 128, 1024);
        const uint32_t d = tbase + kColD + mt * kN;
#pragma unroll
        for (int s = 0; s < kK / 8; ++s) {  // 8 K values per MMA; +256 B per K step
            const uint32_t ah = tbase + kColAhi + mt * kK + s * 8, al = tbase + kColAlo + mt * kK + s * 8;
            mma_tf32_ts(d, ah, dh + (uint64_t)(16 * s), IT, s > 0 ? 1u : 0u);
            mma_tf32_ts(d, ah, dl + (uint64_t)(16 * s), IT, 1u);
            mma_tf32_ts(d, al, dh + (uint64_t)(16 * s), IT, 1u);
        }
        tc::commit(&sm.bar_mma);
    };

    if (nch <= 2) {  // the B operands then stay for every slice
        if (nch > 0) stage_b(0, 0);
        if (nch > 1) stage_b(1, 1);
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tbase = sm.tslot;
    bool ok = true;
    uint32_t mma_par = 0;
    const unsigned gm = 0xfu << (lane & 28);  // the four lanes of a sample
    const int q = wid & 3;                    // TMEM lane quarter of this warp
    // the TMA box is requested by lane 0 of the last warp, the MMAs of M tile
    // mt by lane 0 of warp kWarps - kMT + mt (the last warps: a chunk rarely
    // has enough samples to give them gather work)
    const int issuer = kThr - 32;
    const int imt = (lane == 0 && wid >= kWarps - kMT) ? wid - (kWarps - kMT) : -1;

    // footprint box of slice z -> A operand in tensor memory (thread = cell)
    auto convert = [&](int z) {
        ok = tc::mbar_wait(&sm.bar_tma, (uint32_t)((z - z0) & 1), ok) && ok;
        for (int mt = wid >> 2; mt < kMT; mt += kWarps / 4) {
            const int cell = mt * 128 + 32 * q + lane;
            float hi[32], lo[32];
            if (cell < kCells) {
                const int row = cell / kFW, col = cell - row * kFW;
                const int br = mirrored ? kFW - 1 - row : row, bc = mirrored ? kFW - col : col;
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    const float2 v = sm.box[j][br][bc];
                    hi[2 * j] = v.x;
                    hi[2 * j + 1] = mirrored ? -v.y : v.y;
                }
            } else {
#pragma unroll
                for (int i = 0; i < 32; ++i) hi[i] = 0.f;
            }
#pragma unroll
            for (int i = 0; i < 32; ++i) lo[i] = hi[i] - tc::trunc_tf32(hi[i]);
            const uint32_t ta = tbase + ((uint32_t)(32 * q) << 16);
            st32(ta + kColAhi + mt * kK, hi);
            st32(ta + kColAlo + mt * kK, lo);
        }
        asm volatile("tcgen05.wait::st.sync.aligned;\n" ::: "memory");
        if (nch > 2) {
            stage_b(0, 0);
            stage_b(1, 1);
        }
        tc::fence_proxy_async();
        tc::fence_before();
        __syncthreads();
        if (tid == issuer && z + 1 < z1) tma_issue(z + 1);  // the box buffer has been read
        if (imt >= 0) {
            tc::fence_after();
            issue(tbase, 0, 0, imt);
        }
    };

    if (nch == 0) {  // no samples: only the first box is in flight
        ok = tc::mbar_wait(&sm.bar_tma, 0u, ok) && ok;
    } else {
        convert(z0);
    }
    for (int z = z0; z < z1 && nch > 0; ++z) {
        for (int ch = 0; ch < nch; ++ch) {
            const int nr = min(kRays, nseg - ch * kRays);
            ok = tc::mbar_wait(&sm.bar_mma, mma_par, ok) && ok;
            mma_par ^= 1u;
            tc::fence_after();
            // ---- accumulator -> G (warp w reads TMEM lanes 32 (w % 4) ..):
            // M tiles 0-3 one per group of four warps; tile 4 holds cells in
            // lanes 0-63 only, split four ways by rays (8 columns per warp) ----
            {
                const int mt = wid >> 2;
                float v[32];
                tc::ld32(tbase + ((uint32_t)(32 * q) << 16) + kColD + mt * kN, v);
                const int cell = mt * 128 + 32 * q + lane, gc = cell + cell / kFW;
#pragma unroll
                for (int r = 0; r < kRays; ++r)
                    if (r < nr) sm.g[r][gc] = make_float2(v[2 * r], v[2 * r + 1]);
            }
            static_assert(kMT == 5 && kCells - 4 * 128 <= 64 && kWarps == 16, "G read-out split");
            if (q < 2) {
                const int r0 = 4 * (wid >> 2);  // rays r0 .. r0 + 3
                float v[8];
                tc::ld8(tbase + ((uint32_t)(32 * q) << 16) + kColD + 4 * kN + 2 * r0, v);
                const int cell = 4 * 128 + 32 * q + lane, gc = cell + cell / kFW;
#pragma unroll
                for (int r = 0; r < 4; ++r)
                    if (r0 + r < nr) sm.g[r0 + r][gc] = make_float2(v[2 * r], v[2 * r + 1]);
            }
            tc::fence_before();
            __syncthreads();
            if (ch + 1 < nch) {  // next chunk's MMAs run during this chunk's samples
                if (imt >= 0) {
                    tc::fence_after();
                    issue(tbase, ch + 1, (ch + 1) & 1, imt);
                }
                if (nch > 2 && ch + 2 < nch) {
                    stage_b(ch + 2, ch & 1);
                    tc::fence_proxy_async();
                }
            } else if (z + 1 < z1) {
                // all MMAs of slice z are done: the next slice's A operand and
                // first MMAs go ahead, and run during this chunk's samples
                convert(z + 1);
            }
            // ---- samples of this chunk: four threads per sample (rows p, p+4, p+8) ----
            {
                const int e0 = sm.seg_first[ch * kRays];
                const int e1 = sm.seg_first[min((ch + 1) * kRays, nseg)];
                const int part = tid & 3;
                for (int t = tid >> 2; e0 + t < e1; t += kThr / 4) {
                    const int e = e0 + t;
                    const int pos = sm.pos[e];
                    const float2 *gp = sm.g[sm.seg_of[e] - ch * kRays] + (pos < 0 ? 0 : pos);
                    float ex[kTaps];
#pragma unroll
                    for (int b = 0; b < kTaps; ++b) ex[b] = sm.wx[e][b];
                    float2 acc2 = make_float2(0.f, 0.f);
#pragma unroll
                    for (int i = 0; i < 3; ++i) {
                        const int a = part + 4 * i;
                        if (a < kTaps) {
                            const float2 *gr = gp + a * kGP;
                            float2 rr = make_float2(0.f, 0.f);
#pragma unroll
                            for (int b = 0; b < kTaps; ++b) rr = ffma2(make_float2(ex[b], ex[b]), gr[b], rr);
                            const float wy = sm.wy[e][a];
                            acc2 = ffma2(make_float2(wy, wy), rr, acc2);
                        }
                    }
                    float ax = acc2.x, ay = acc2.y;
                    ax += __shfl_xor_sync(gm, ax, 1);
                    ay += __shfl_xor_sync(gm, ay, 1);
                    ax += __shfl_xor_sync(gm, ax, 2);
                    ay += __shfl_xor_sync(gm, ay, 2);
                    if (part == 0 && pos >= 0) {
                        const int th = sm.th[e], k = sm.k[e];
                        float2 r = cmul(make_float2(ax, ay), sm.f[e]);
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
            __syncthreads();
        }
    }
    tc::fence_before();
    __syncthreads();
    if (wid == 0) tc::dealloc(tbase, kTmemCols);
    if (!ok && lane == 0) atomicAdd(err, 1);
}

size_t gather_tc_smem() { return sizeof(TcSmem); }

void gather_tc_prepare() {
    CUDA_CHECK(cudaFuncSetAttribute(k_gather_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)sizeof(TcSmem)));
}

void make_spec_tensor_map(CUtensorMap *map, float2 *spec, int nimg, const UsGeo &g) {
    static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    if (!encode) {
        cudaDriverEntryPointQueryResult q;
        CUDA_CHECK(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", (void **)&encode, 12000,
                                                    cudaEnableDefault, &q));
        if (q != cudaDriverEntryPointSuccess || !encode) throw Error(1, "cuTensorMapEncodeTiled unavailable");
    }
    // float view: [images][P + 2 kHalo rows][2 qp floats]
    const cuuint64_t dims[3] = {(cuuint64_t)2 * g.qp, (cuuint64_t)(g.P + 2 * kHalo), (cuuint64_t)nimg};
    const cuuint64_t strides[2] = {(cuuint64_t)g.qp * 8, (cuuint64_t)g.img_fwd * 8};
    const cuuint32_t box[3] = {2 * kBoxW, kFW, 16};
    const cuuint32_t es[3] = {1, 1, 1};
    const CUresult r = encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, spec, dims, strides, box, es,
                              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) throw Error(1, "cuTensorMapEncodeTiled failed for the forward spectra");
}

void launch_gather_tc(float2 *rows, int zb, const GeoDev &gd, const UsGeo &g, const CUtensorMap &tmap, int jbase,
                      int accumulate, cudaStream_t s) {
    if (gd.n_fwd_tc_items == 0) return;
    if (g.T != kT) throw Error(1, "tile size must be 16");
    if (g.zper < 1 || g.zper > kZPer) throw Error(1, "gather slices per block must be in [1, 64]");
    dim3 gs(gd.n_fwd_tc_items, (zb + g.zper - 1) / g.zper);
    k_gather_tc<<<gs, kThr, sizeof(TcSmem), s>>>(rows, gd.fwd_pts, gd.fwd_tc_items, gd.sincos, gd.kmat, gd.shiftfwd,
                                                 tmap, g, zb, jbase, accumulate, gd.err);
    LAUNCH_CHECK("k_gather_tc");
}

int gather_tc_table_capacity() { return kTab; }

}  // namespace rectv
