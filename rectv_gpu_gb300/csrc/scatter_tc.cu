// Adjoint USFFT scatter with the time-sample mixing on the tensor cores
// (tcgen05).
//
// The adjoint (gather TOMO_ADJ + wrap TOMO_ADJ, kernels_radonusfft.cuh:40-144,
// fused with shift/fftshift of radonusfft.cu:115-121 and the basis weights of
// operators.cu:171-176) adds, for every polar sample p on ray theta, the value
// conj(K'(theta, j)) w(p, c) E(p) to cell c of time sample j's grid, with the
// separable Gaussian weight w(p, c) = wx_p(cx) wy_p(cy).
//
// Geometry records.  The weights of a sample restricted to one 16x16 tile
// do not depend on the slice, so they are computed once per geometry
// (k_adj_records) for every (tile, sample) entry of the adjoint plan: the
// x and y weight rows over the tile's 16 columns / rows (zero outside the
// stencil), the ray, the detector index and a mask of the tile rows the
// stencil covers.
//
// Tables.  A tile's entries are cut into tables of whole rays, at most one
// MMA batch of rays (16) and 256 entries each (host plan); the ray
// segmentation of a table (its rays, their first rows, and per ray and warp
// the rows covering the warp's two tile rows) is geometry too, computed once
// by k_adj_tabinfo.
//
// Persistent blocks of 512 threads, one per SM, take the (tile, slice pair)
// units with samples round-robin; each block half (256 threads, thread =
// cell) works on one slice of the pair, and the halves share what does not
// depend on the slice: the records, the segmentation, K' (the MMA's B) and
// the barriers.  The records and segmentation of the next table are
// bulk-copied into a second shared buffer (TMA engine, mbarrier) while the
// current one is processed.  Per unit and table:
//  * per entry: E(p) (the row spectrum value times (-1)^(k+1) shiftadj(k)
//    (pi/mu)/n) of both slices and T_p(cy) = E(p) wy_p(cy) for the tile's 16
//    rows, both slices in one float4;
//  * per batch of 16 rays: every cell sums its value of each ray's grid
//    V(c, theta) = sum_p T_p(cy) wx_p(cx) over the ray's samples (plan order,
//    so sums are reproducible; a warp skips samples that miss its two rows);
//    the time samples are then a GEMM over the batch's rays,
//    F(c, j) += sum_theta V(c, theta) conj(K'(theta, j)), [256 x 32] x
//    [32 x 32] real on the tensor cores with TF32 parts for FP32 accuracy
//    (the tensor core truncates FP32 input to TF32; lo = x - trunc(x)):
//    the MMA's B holds [Khi | Klo] as 64 columns, so Vhi B + Vlo B gives
//    Vhi Khi + Vhi Klo + Vlo Khi (+ the negligible Vlo Klo) in 16 MMAs.
//    Each batch's product is added to the cell's FP32 sums in registers (the
//    tensor core's own FP32 accumulation rounds differently and would drift
//    over the many batches of central tiles), and the next table's E and T
//    and ray sums are formed while the MMAs run.
// The tile is added once per unit into the Hermitian half plane that the
// C2R inverse transform takes (see the epilogue).
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>

#include "rectv_internal.cuh"
#include "tcgen05.cuh"
#include "usfft_common.cuh"

namespace rectv {

namespace {

constexpr int kT = 16;
constexpr int kCells = kT * kT;     // 256 = 2 M tiles
constexpr int kMT = kCells / 128;
constexpr int kZ = 2;               // slices per unit: one per block half
constexpr int kTab = 256;           // samples per table
constexpr int kBatch = 16;          // rays per MMA batch (K = 32)
constexpr int kK = 2 * kBatch;
constexpr int kN = 32;              // 16 time samples x (re, im)
constexpr int kNP = 2 * kN;         // MMA N: B rows [Khi | Klo]
constexpr int kHalf = kCells;       // threads per slice: one per cell
constexpr int kThr = kZ * kHalf;    // 512
constexpr int kHW = kHalf / 32;     // warps per half: warp w covers tile rows 2w, 2w+1
constexpr uint32_t kSliceCols = 256;           // TMEM columns of one slice:
constexpr uint32_t kColAhi = 0;                //   A hi [mt*32, +32)
constexpr uint32_t kColAlo = kMT * kK;         //   A lo (64)
constexpr uint32_t kColD = 2 * kMT * kK;       //   product of the batch [128 + mt*64, +64)
constexpr uint32_t kTmemCols = kZ * kSliceCols;  // 512: the whole SM (one block per SM)
static_assert(kTab <= kHalf, "one table entry per thread of a half");

__device__ __forceinline__ int off32(int row, int kk) {
    return (row >> 3) * 256 + (kk >> 2) * 32 + (row & 7) * 4 + (kk & 3);
}

// 32-bit words of a table's ray segmentation (adj_info_words; an empty range
// is lo = kTab, hi = 0)
constexpr int info_words(int nseg) { return adj_info_words(nseg); }
constexpr int kInfoMax = info_words(kTab);

struct ScTcSmem {
    AdjRec rec[2][kTab];          // geometry records of this table and the next (bulk copies)
    uint32_t info[2][kInfoMax];   // their ray segmentation (bulk copies)
    float4 t[kT][kTab];           // T_p(cy) = E(p) wy_p(cy) of both slices of the pair (x, y | z, w)
    float4 rnext[kZ][kTab];       // row spectrum values of the next table's samples, both slices (cp.async;
                                  // each half copies its own, so a thread reads only its own copies)
    float bhi[kN * kK];           // B = conj K' of the batch's rays, FP32: rows 0..31 of the MMA's B
    float blo[kN * kK];           // B - trunc(B): rows 32..63 (contiguous with bhi)
    unsigned long long bar;      // MMA batch done (both slices)
    unsigned long long rbar[2];  // record buffer landed
    uint32_t tslot;
};

__device__ __forceinline__ void st16(uint32_t taddr, const float (&v)[16]) {
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};\n" ::"r"(
            taddr),
        "f"(v[0]), "f"(v[1]), "f"(v[2]), "f"(v[3]), "f"(v[4]), "f"(v[5]), "f"(v[6]), "f"(v[7]), "f"(v[8]), "f"(v[9]),
        "f"(v[10]), "f"(v[11]), "f"(v[12]), "f"(v[13]), "f"(v[14]), "f"(v[15])
        : "memory");
}

__device__ __forceinline__ void mma_tf32_ts(uint32_t d, uint32_t a, uint64_t b, uint32_t id, uint32_t acc) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n}\n" ::"r"(d),
        "r"(a), "l"(b), "r"(id), "r"(acc)
        : "memory");
}

}  // namespace

// ---------------------------------------------------------------------------
// Geometry records of the adjoint plan: one block per work item, one thread
// per entry.  The stencil origin is taken modulo the periodic grid nearest to
// the tile (wrap TOMO_ADJ, kernels_radonusfft.cuh:40-64).
// ---------------------------------------------------------------------------
__global__ void k_adj_records(AdjRec *__restrict__ recs, const uint32_t *__restrict__ pts,
                              const int4 *__restrict__ items, const float2 *__restrict__ sincos,
                              const float2 *__restrict__ shifta, UsGeo g) {
    const int4 it = items[blockIdx.x];
    const int tyi = it.x / g.NT, txi = it.x - tyi * g.NT;
    const int P = g.P, half = P / 2;
    for (int e = threadIdx.x; e < it.z; e += blockDim.x) {
        const uint32_t id = pts[it.y + e];
        const int th = id / (uint32_t)g.n;
        const int k = id - th * g.n;
        float x0, y0;
        int fx, fy;
        sample_pos(k, sincos[th], g, x0, y0, fx, fy);
        int dx = g.n + fx - kR - txi * kT;
        int dy = g.n + fy - kR - tyi * kT;
        dx += (dx < -half) ? P : 0;
        dx -= (dx > half) ? P : 0;
        dy += (dy < -half) ? P : 0;
        dy -= (dy > half) ? P : 0;
        AdjRec r;
        int mask = 0;
#pragma unroll
        for (int c = 0; c < kT; ++c) {
            const int bx = c - dx, by = c - dy;
            r.wx[c] = ((unsigned)bx < (unsigned)kTaps) ? tap_weight(fx, bx, x0, g) : 0.f;
            const bool iny = (unsigned)by < (unsigned)kTaps;
            r.wy[c] = iny ? tap_weight(fy, by, y0, g) : 0.f;
            mask |= iny ? (1 << c) : 0;
        }
        r.thm = (th << 16) | mask;
        r.k = k;
        const float2 sh = shifta[k];
        const float cf = (k & 1) ? g.cw : -g.cw;
        r.sf = make_float2(sh.x * cf, sh.y * cf);
        recs[(long long)it.y + e] = r;
    }
}

void launch_adj_records(AdjRec *recs, const GeoDev &gd, const UsGeo &g, cudaStream_t s) {
    if (gd.n_adj_items == 0) return;
    k_adj_records<<<gd.n_adj_items, 256, 0, s>>>(recs, gd.adj_pts, gd.adj_items, gd.sincos, gd.shiftadj, g);
    LAUNCH_CHECK("k_adj_records");
}

// ---------------------------------------------------------------------------
// Ray segmentation of every scatter table (geometry only, so computed once):
// the rays (runs of equal theta, records are theta-major), their first rows,
// and per ray and warp of a block half the rows [lo, hi) from the first to
// the last sample whose stencil covers the warp's two tile rows, from the
// samples where a covered run starts or ends.  One block per table.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kTab)
    k_adj_tabinfo(const AdjRec *__restrict__ recs, const int4 *__restrict__ tabs, uint32_t *__restrict__ info) {
    __shared__ int seg_first[kTab + 1];
    __shared__ int rlo[kHW][kTab], rhi[kHW][kTab];
    __shared__ int wsum[kTab / 32];
    const int4 tb = tabs[blockIdx.x];  // (first entry, count, word offset, words)
    const int ct = threadIdx.x, lane = ct & 31, w = ct >> 5, cnt = tb.y;
    int thm = 0, thp = 0, thn = 0;
    if (ct < cnt) {
        thm = recs[(long long)tb.x + ct].thm;
        if (ct > 0) thp = recs[(long long)tb.x + ct - 1].thm;
        if (ct + 1 < cnt) thn = recs[(long long)tb.x + ct + 1].thm;
    }
    const unsigned th = (unsigned)thm >> 16;
    const int flag = (ct < cnt && (ct == 0 || ((unsigned)thp >> 16) != th)) ? 1 : 0;
    int incl = flag;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) wsum[w] = incl;
    __syncthreads();
    int base = 0, nseg = 0;
#pragma unroll
    for (int i = 0; i < kTab / 32; ++i) {
        base += (i < w) ? wsum[i] : 0;
        nseg += wsum[i];
    }
    const int seg = incl + base - 1;
    if (ct < cnt && flag) {
        seg_first[seg] = ct;
#pragma unroll
        for (int i = 0; i < kHW; ++i) {
            rlo[i][seg] = kTab;
            rhi[i][seg] = 0;
        }
    }
    if (ct == 0) seg_first[nseg] = cnt;
    __syncthreads();
    if (ct < cnt) {
        const int msk = thm & 0xffff;
        const int mprev = flag ? 0 : (thp & 0xffff);
        const bool last = ct + 1 == cnt || ((unsigned)thn >> 16) != th;
        const int mnext = last ? 0 : (thn & 0xffff);
#pragma unroll
        for (int i = 0; i < kHW; ++i) {
            const int bits = 3 << (2 * i);
            if (msk & bits) {
                if (!(mprev & bits)) atomicMin(&rlo[i][seg], ct);
                if (!(mnext & bits)) atomicMax(&rhi[i][seg], ct + 1);
            }
        }
    }
    __syncthreads();
    uint32_t *out = info + tb.z;
    const int nw = min(info_words(nseg), tb.w);  // the host sized the slot from the same rays
    for (int i = ct; i < nw; i += kTab) {
        uint32_t v = 0;
        if (i == 0) {
            v = (uint32_t)nseg;
        } else if (i >= 4 && i < 4 + 8 * nseg) {
            const int sg = (i - 4) >> 3, ww = (i - 4) & 7;
            v = (uint32_t)rlo[ww][sg] | ((uint32_t)rhi[ww][sg] << 16);
        } else if (i >= 4 + 8 * nseg) {
            const int j = 2 * (i - 4 - 8 * nseg);  // 16-bit ray starts j, j+1
            if (j <= nseg) v = (uint32_t)seg_first[j];
            if (j + 1 <= nseg) v |= (uint32_t)seg_first[j + 1] << 16;
        }
        out[i] = v;
    }
}

int scatter_tc_table_capacity() { return kTab; }
int scatter_tc_batch_rays() { return kBatch; }
int scatter_tc_info_words(int nseg) { return info_words(nseg); }

void launch_adj_tabinfo(const GeoDev &gd, cudaStream_t s) {
    if (gd.n_adj_tabs == 0) return;
    k_adj_tabinfo<<<gd.n_adj_tabs, kTab, 0, s>>>(gd.adj_recs, gd.adj_tabs, gd.adj_info);
    LAUNCH_CHECK("k_adj_tabinfo");
}

__global__ void __launch_bounds__(kThr, 1)
    k_scatter_tc(const float2 *__restrict__ rowsc, float2 *__restrict__ spec, const AdjRec *__restrict__ recs,
                 const int4 *__restrict__ items, const int4 *__restrict__ tabs, const int *__restrict__ tab_base,
                 const uint32_t *__restrict__ info, const float2 *__restrict__ kmat,
                 const float2 *__restrict__ shifta, UsGeo g, int zb, int npairs, int nunits, int jbase,
                 int *__restrict__ err) {
    extern __shared__ __align__(1024) unsigned char sc_smem_raw[];
    ScTcSmem &sm = *reinterpret_cast<ScTcSmem *>(sc_smem_raw);
    const int P = g.P, hn = g.n / 2 + 1;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int h = tid / kHalf;     // block half: slice 2 pair + h
    const int ct = tid % kHalf;    // this thread's cell ct = mt*128 + 32q + lane
    const int hw = wid % kHW;      // warp within the half (tile rows 2hw, 2hw+1)
    if (wid == 0) tc::alloc(&sm.tslot, kTmemCols);
    if (tid == 0) {
        tc::mbar_init(&sm.bar, kZ * kMT);  // one commit per (slice, M tile) chain
        tc::mbar_init(&sm.rbar[0], 1);
        tc::mbar_init(&sm.rbar[1], 1);
        tc::fence_mbar_init();
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tbase = sm.tslot;
    const uint32_t tsl = tbase + h * kSliceCols;  // this slice's TMEM columns
    const int mt = ct >> 7, q = wid & 3;          // TMEM lane quarter of this warp
    const int cx = ct % kT, cy = ct / kT;
    bool ok = true;
    int nmma = 0;  // MMA batches issued by this block (phase of sm.bar)
    int seq = 0;   // tables consumed: buffer seq & 1, its fill (seq >> 1) & 1
    // Thread 0's copy cursor: the next table (unit, first entry) to fetch, in
    // the order the tables are consumed; a table is fetched while the one
    // before it is processed.
    int fu = blockIdx.x, ft = 0;
    auto fetch = [&](int slot) {  // records and segmentation of table ft of unit fu
        if (fu >= nunits) return;
        const int item = fu / npairs;
        const int tb0 = __ldg(tab_base + item), tb1 = __ldg(tab_base + item + 1);
        const int4 tb = __ldg(tabs + tb0 + ft);
        const uint32_t rbytes = (uint32_t)tb.y * (uint32_t)sizeof(AdjRec), ibytes = (uint32_t)tb.w * 4u;
        const uint32_t bar = tc::smem_addr(&sm.rbar[slot]);
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"(rbytes + ibytes)
                     : "memory");
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                         tc::smem_addr(sm.rec[slot])),
                     "l"(recs + tb.x), "r"(rbytes), "r"(bar)
                     : "memory");
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                         tc::smem_addr(sm.info[slot])),
                     "l"(info + tb.z), "r"(ibytes), "r"(bar)
                     : "memory");
        if (++ft >= tb1 - tb0) {
            ft = 0;
            fu += gridDim.x;
        }
    };
    if (tid == 0) fetch(0);
    bool have_next = false;  // rnext holds the current table's row spectrum values (both slices)

    // persistent: units (tile item, slice pair) round-robin, pairs fastest, so
    // the blocks in flight share their items' records in L2; all units hold
    // samples.  The two halves share the records, ray starts, sample ranges and
    // K' (B); each has its slice's E, T, A, accumulator and sums.
    for (int u = blockIdx.x; u < nunits; u += gridDim.x) {
        const int z = 2 * (u % npairs) + h;
        const bool zok = z < zb;  // the last pair of an odd batch has one slice
        const int4 it = __ldg(items + u / npairs);
        const int tyi = it.x / g.NT, txi = it.x - tyi * g.NT;
        int nbu = 0;    // MMA batches of this unit
        float acc[32];  // F of this cell: 16 time samples x (re, im)
#pragma unroll
        for (int i = 0; i < 32; ++i) acc[i] = 0.f;

        const int tb0 = __ldg(tab_base + u / npairs), tb1 = __ldg(tab_base + u / npairs + 1);
        for (int ti = tb0; ti < tb1; ++ti) {
            const int cnt = __ldg(tabs + ti).y;
            const int buf = seq & 1;
            // the other record buffer and T are free: every thread has passed
            // the barrier in front of the previous table's MMAs, after its ray sums
            if (tid == 0) {
                tc::fence_proxy_async();
                fetch(buf ^ 1);
            }
            ok = tc::mbar_wait(&sm.rbar[buf], (uint32_t)((seq >> 1) & 1), ok) && ok;
            ++seq;
            const AdjRec *rec = sm.rec[buf];
            const uint32_t *inf = sm.info[buf];
            const int nseg = min((int)inf[0], cnt);  // (clamps keep every index inside the table)
            const uint16_t *segf = reinterpret_cast<const uint16_t *>(inf + 4 + 8 * nseg);  // ray starts
            // ---- E = (-1)^(k+1) shiftadj(k) FFT(row)(k) (pi/mu)/n of both slices and
            // T_p(cy) = E(p) wy_p(cy), stored [row][entry] as float4 (slice 0 | slice 1):
            // thread (h, e) writes rows 8h .. 8h+7 of entry e ----
            if (have_next) asm volatile("cp.async.wait_all;\n" ::: "memory");  // this thread's own copies
            if (ct < cnt) {
                const int th = (unsigned)rec[ct].thm >> 16, k = rec[ct].k;
                float4 R = make_float4(0.f, 0.f, 0.f, 0.f);
                if (have_next) {
                    R = sm.rnext[h][ct];
                } else {
                    const long long o = (long long)th * hn + (k <= g.n / 2 ? k : g.n - k);
                    const int z0 = 2 * (u % npairs);
                    if (z0 < zb) {
                        const float2 r0 = __ldg(rowsc + (long long)z0 * g.ntheta * hn + o);
                        R.x = r0.x;
                        R.y = r0.y;
                    }
                    if (z0 + 1 < zb) {
                        const float2 r1 = __ldg(rowsc + (long long)(z0 + 1) * g.ntheta * hn + o);
                        R.z = r1.x;
                        R.w = r1.y;
                    }
                }
                if (k > g.n / 2) {
                    R.y = -R.y;
                    R.w = -R.w;
                }
                const float2 sf = rec[ct].sf;
                const float2 E0 = cmul(make_float2(R.x, R.y), sf), E1 = cmul(make_float2(R.z, R.w), sf);
                const float4 *wy4 = reinterpret_cast<const float4 *>(rec[ct].wy) + 2 * h;  // rows 8h ..
#pragma unroll
                for (int q4 = 0; q4 < 2; ++q4) {
                    const float4 w = wy4[q4];
                    const int r0 = 8 * h + 4 * q4;
                    sm.t[r0 + 0][ct] = make_float4(E0.x * w.x, E0.y * w.x, E1.x * w.x, E1.y * w.x);
                    sm.t[r0 + 1][ct] = make_float4(E0.x * w.y, E0.y * w.y, E1.x * w.y, E1.y * w.y);
                    sm.t[r0 + 2][ct] = make_float4(E0.x * w.z, E0.y * w.z, E1.x * w.z, E1.y * w.z);
                    sm.t[r0 + 3][ct] = make_float4(E0.x * w.w, E0.y * w.w, E1.x * w.w, E1.y * w.w);
                }
            }
            __syncthreads();

            for (int sb = 0; sb < nseg; sb += kBatch) {
                const int nb = min(kBatch, nseg - sb);
                // K'(ray, j) of this thread's two B entries (half 0), loaded before
                // the ray sums so that the L2 latency is not in front of the barrier
                const int brow = ct >> 3, bq4 = ct & 7;  // B row 2j+o, K values 4 bq4 .. 4 bq4 + 3
                const int bj = brow >> 1;
                float2 kv[2];
#pragma unroll
                for (int i = 0; i < 2; ++i) {
                    const int r = 2 * bq4 + i;
                    kv[i] = make_float2(0.f, 0.f);
                    if (h == 0 && r < nb && jbase + bj < g.m)
                        kv[i] = __ldg(kmat + (long long)((unsigned)rec[min((int)segf[sb + r], cnt - 1)].thm >> 16) * g.m +
                                      jbase + bj);
                }
                // ---- 1. V(c, ray) of this cell for rays [8h, 8h + 8) of the
                // batch, both slices of the pair (one weight load, one T load, two FMAs) ----
                constexpr int kRH = kBatch / kZ;  // rays per half
                float v0[2 * kRH], v1[2 * kRH];
#pragma unroll
                for (int r = 0; r < kRH; ++r) {
                    const int rr = kRH * h + r;
                    float2 a = make_float2(0.f, 0.f), b = make_float2(0.f, 0.f);
                    if (rr < nb) {  // T and wx vanish outside the stencil: no tests in the loop
                        const uint32_t lohi = inf[4 + 8 * (sb + rr) + hw];
                        const int e1 = min((int)(lohi >> 16), cnt);
#pragma unroll 4
                        for (int e = (int)(lohi & 0xffffu); e < e1; ++e) {
                            const float w = rec[e].wx[cx];
                            const float4 tv = sm.t[cy][e];  // both slices in one load
                            a = ffma2(make_float2(w, w), make_float2(tv.x, tv.y), a);
                            b = ffma2(make_float2(w, w), make_float2(tv.z, tv.w), b);
                        }
                    }
                    v0[2 * r] = a.x;
                    v0[2 * r + 1] = a.y;
                    v1[2 * r] = b.x;
                    v1[2 * r + 1] = b.y;
                }
                // ---- the next table's row spectrum values, copied while this
                // table's batches run: after the first batch's ray sums, by
                // which time the next records (fetched at this table's start) have landed ----
                if (sb == 0) {
                    int nti = ti + 1, nu = u;
                    if (nti >= tb1) {
                        nu = u + gridDim.x;
                        nti = nu < nunits ? __ldg(tab_base + nu / npairs) : 0;
                    }
                    have_next = nu < nunits;
                    if (have_next) {
                        const int ncnt = __ldg(tabs + nti).y;
                        const int nz0 = 2 * (nu % npairs);  // both slices of the next unit's pair
                        ok = tc::mbar_wait(&sm.rbar[buf ^ 1], (uint32_t)((seq >> 1) & 1), ok) && ok;
                        if (ct < ncnt) {
                            const AdjRec &nr = sm.rec[buf ^ 1][ct];
                            const int th = (unsigned)nr.thm >> 16, k = nr.k;
                            const long long o = (long long)th * hn + (k <= g.n / 2 ? k : g.n - k);
                            float2 *dst = reinterpret_cast<float2 *>(&sm.rnext[h][ct]);
                            if (nz0 < zb)
                                asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(tc::smem_addr(dst)),
                                             "l"(rowsc + (long long)nz0 * g.ntheta * hn + o)
                                             : "memory");
                            else
                                dst[0] = make_float2(0.f, 0.f);
                            if (nz0 + 1 < zb)
                                asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(tc::smem_addr(dst + 1)),
                                             "l"(rowsc + (long long)(nz0 + 1) * g.ntheta * hn + o)
                                             : "memory");
                            else
                                dst[1] = make_float2(0.f, 0.f);
                            asm volatile("cp.async.commit_group;\n" ::: "memory");
                        }
                    }
                }
                // ---- previous batch's MMAs done: add its product to the cell's
                // FP32 sums; A, B and the accumulator are then free ----
                if (nbu > 0) {
                    ok = tc::mbar_wait(&sm.bar, (uint32_t)((nmma - 1) & 1), ok) && ok;
                    tc::fence_after();
                    float v[32], w2[32];
                    tc::ld32(tsl + ((uint32_t)(32 * q) << 16) + kColD + mt * kNP, v);
                    tc::ld32(tsl + ((uint32_t)(32 * q) << 16) + kColD + mt * kNP + kN, w2);
#pragma unroll
                    for (int i = 0; i < 32; ++i) acc[i] += v[i] + w2[i];
                }
                // ---- B = conj K' rows of this batch: row 2j+o, K index 2r+s (half 0: threads = (row, 4 K values)) ----
                if (h == 0) {
                    const int o = brow & 1;
                    float bv[4];
#pragma unroll
                    for (int i = 0; i < 2; ++i) {
                        bv[2 * i] = o == 0 ? kv[i].x : -kv[i].y;
                        bv[2 * i + 1] = o == 0 ? kv[i].y : kv[i].x;
                    }
                    const int o32 = off32(brow, 4 * bq4);
                    *reinterpret_cast<float4 *>(sm.bhi + o32) = make_float4(bv[0], bv[1], bv[2], bv[3]);
                    *reinterpret_cast<float4 *>(sm.blo + o32) =
                        make_float4(bv[0] - tc::trunc_tf32(bv[0]), bv[1] - tc::trunc_tf32(bv[1]),
                                    bv[2] - tc::trunc_tf32(bv[2]), bv[3] - tc::trunc_tf32(bv[3]));
                }
                // ---- 2. A = V of this cell, hi and lo parts, into tensor memory:
                // K columns 16h .. 16h + 15 (this half's rays) of both slices ----
                {
                    float lo[2 * kRH];
                    const uint32_t ta0 = tbase + ((uint32_t)(32 * q) << 16) + mt * kK + 2 * kRH * h;
#pragma unroll
                    for (int i = 0; i < 2 * kRH; ++i) lo[i] = v0[i] - tc::trunc_tf32(v0[i]);
                    st16(ta0 + kColAhi, v0);
                    st16(ta0 + kColAlo, lo);
#pragma unroll
                    for (int i = 0; i < 2 * kRH; ++i) lo[i] = v1[i] - tc::trunc_tf32(v1[i]);
                    st16(ta0 + kSliceCols + kColAhi, v1);
                    st16(ta0 + kSliceCols + kColAlo, lo);
                    asm volatile("tcgen05.wait::st.sync.aligned;\n" ::: "memory");
                }
                tc::fence_proxy_async();
                tc::fence_before();
                __syncthreads();
                // one issuing thread per (slice, M tile) accumulator chain: lane 0
                // of the last two warps of each half, whose table entries (rows
                // 192-255) are idle in the next table's E/T phase for most tables
                constexpr int iw = kHW - 2;
                if (lane == 0 && (hw == iw || hw == iw + 1)) {
                    tc::fence_after();
                    // D = [Ahi Bhi, Ahi Blo] + [Alo Bhi, Alo Blo]: both halves summed when read
                    constexpr uint32_t IT = tc::idesc(tc::kFmtTF32, 128, kNP);
                    const uint64_t db = tc::sdesc(tc::smem_addr(sm.bhi), 128, 1024);
                    const int m2 = hw - iw;
                    const uint32_t d = tsl + kColD + m2 * kNP;
#pragma unroll
                    for (int s2 = 0; s2 < kK / 8; ++s2) {
                        const uint32_t ah = tsl + kColAhi + m2 * kK + s2 * 8;
                        const uint32_t al = tsl + kColAlo + m2 * kK + s2 * 8;
                        mma_tf32_ts(d, ah, db + (uint64_t)(16 * s2), IT, s2 > 0 ? 1u : 0u);
                        mma_tf32_ts(d, al, db + (uint64_t)(16 * s2), IT, 1u);
                    }
                    tc::commit(&sm.bar);
                }
                ++nmma;
                ++nbu;
            }
        }
        // ---- the unit's last product ----
        if (nbu > 0) {
            ok = tc::mbar_wait(&sm.bar, (uint32_t)((nmma - 1) & 1), ok) && ok;
            tc::fence_after();
            float v[32], w2[32];
            tc::ld32(tsl + ((uint32_t)(32 * q) << 16) + kColD + mt * kNP, v);
            tc::ld32(tsl + ((uint32_t)(32 * q) << 16) + kColD + mt * kNP + kN, w2);
#pragma unroll
            for (int i = 0; i < 32; ++i) acc[i] += v[i] + w2[i];
        }
        // ---- the adjoint only needs Re IFFT2(X) = C2R of the Hermitian part
        // H(k) = (X(k) + conj X(-k)) / 2 on the half plane kx <= n: each cell adds
        // X(k)/2 to H(k) and conj(X(k))/2 to H(-k) where they lie in the half plane
        // (at most two adds per H cell from two blocks, onto zeros: the sum does not
        // depend on their order); the pre-IFFT fftshift sign is applied here ----
        const int KY = tyi * kT + cy, KX = txi * kT + cx;
        if (zok && KY < P && KX < P) {
            const int half = P / 2, hp = g.hpitch;
            const long long img_half = (long long)P * hp;
            const float sg = ((KX + KY) & 1) ? -0.5f : 0.5f;
            const bool here = KX <= half, mirror = KX >= half || KX == 0;
            const long long o1 = (long long)KY * hp + KX;
            const long long o2 = (long long)((P - KY) % P) * hp + (P - KX) % P;
            float2 *dst = spec + ((long long)z * g.m + jbase) * img_half;
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                if (jbase + j >= g.m) break;
                const float2 v = make_float2(sg * acc[2 * j], sg * acc[2 * j + 1]);
                float2 *d = dst + (long long)j * img_half;
                if (here) atomicAdd(d + o1, v);
                if (mirror) atomicAdd(d + o2, make_float2(v.x, -v.y));
            }
        }
    }  // units
    tc::fence_before();
    __syncthreads();
    if (wid == 0) tc::dealloc(tbase, kTmemCols);
    if (!ok && lane == 0) atomicAdd(err, 1);
}

// One block per SM: it holds all 512 tensor-memory columns (two slices x 256).
constexpr size_t kScSmemBytes = sizeof(ScTcSmem);

void scatter_tc_prepare() {
    CUDA_CHECK(cudaFuncSetAttribute(k_scatter_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kScSmemBytes));
}

void launch_scatter_tc(const float2 *rowsc, float2 *spec, int zb, const GeoDev &gd, const UsGeo &g, int jbase,
                       cudaStream_t s) {
    if (g.T != kT) throw Error(1, "tile size must be 16");
    if (!gd.adj_recs) throw Error(1, "adjoint geometry records missing");
    // items with samples (sorted by count, so the empty tiles, whose half
    // planes stay zero, come last), times slice pairs
    const int npairs = (zb + kZ - 1) / kZ;
    const long long nunits = (long long)npairs * gd.n_adj_busy;
    if (nunits == 0) return;
    if (nunits > 2147483647LL) throw Error(1, "adjoint grid too large");
    static int nsm = 0;
    if (nsm == 0) {
        int dev = 0;
        CUDA_CHECK(cudaGetDevice(&dev));
        CUDA_CHECK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    }
    const int grid = (int)std::min<long long>(nunits, g.sc_grid > 0 ? g.sc_grid : nsm);
    if (!gd.adj_tabs || !gd.adj_info) throw Error(1, "adjoint table segmentation missing");
    k_scatter_tc<<<grid, kThr, kScSmemBytes, s>>>(rowsc, spec, gd.adj_recs, gd.adj_items, gd.adj_tabs,
                                                  gd.adj_tab_base, gd.adj_info, gd.kmat, gd.shiftadj, g, zb, npairs,
                                                  (int)nunits, jbase, gd.err);
    LAUNCH_CHECK("k_scatter_tc");
}

}  // namespace rectv
