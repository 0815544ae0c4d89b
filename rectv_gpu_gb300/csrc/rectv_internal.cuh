// Internal declarations shared by the CUDA translation units of librectv_gb300.
//
// Data layout in HBM (all float32 unless stated):
//   volume  u  [z][t][y][x]            z < nz, t < m (time samples), y,x < n
//   data    g  [z][theta][s]           s < n (detector)
//   dual    psi, mu: SoA [4][chunk][qz][qt][qy][qx], qz<=nzp, qt<=m, qy,qx<=n
//   spectra half-plane R2C images [z][t][P][P/2+1] complex (forward) or full
//           periodic planes [z][t][P][P] complex (adjoint), P = 2n
//   rows    [z][theta][n] complex (forward), [z][theta][n+2] real / n/2+1
//           complex in-place R2C (adjoint)
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <cufft.h>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

namespace rectv {

// USFFT interpolation radius.  radonusfft.cu:11 evaluates to 4 for every n;
// kernels are specialised for it and the host checks the formula.
constexpr int kR = 4;
constexpr int kTaps = 2 * kR + 1;
// halo of the stored forward spectra (see UsGeo::qp)
constexpr int kHalo = 24;
// The USFFT kernels of the reference use this truncated value of pi
// (kernels_radonusfft.cuh:1).
constexpr double kPiUsfft = 3.1415926535;

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

void cuda_check(cudaError_t e, const char *what, const char *file, int line);
void cufft_check(cufftResult e, const char *what, const char *file, int line);
#define CUDA_CHECK(x) ::rectv::cuda_check((x), #x, __FILE__, __LINE__)
#define CUFFT_CHECK(x) ::rectv::cufft_check((x), #x, __FILE__, __LINE__)
#define LAUNCH_CHECK(what) ::rectv::cuda_check(cudaGetLastError(), what, __FILE__, __LINE__)

// Geometry of the USFFT kernels.
struct UsGeo {
    int n, ntheta, m;   // detector width, projections, time samples
    int P;              // oversampled grid side 2n
    int hp;             // half-plane row length P/2+1 (complex)
    int hpitch;         // row pitch of the adjoint's Hermitian half planes (complex):
                        // P/2+1, or P/2+2 (16-byte rows for TMA) with the padded-grid FFTs
    // Forward spectra are stored as the window rows [-kHalo, P+kHalo) x
    // columns [-kHalo, n+kHalo) of the periodic full spectrum: the R2C output
    // (rows [0,P), columns [0,n]) plus a halo of wrapped / Hermitian-mirrored
    // cells, so that every tile footprint is one rectangular box.
    int qp;             // row pitch of a forward image (complex), even
    long long qoff;     // offset of cell (0, 0) in a forward image
    long long img_fwd;  // complex elements per forward image ((P + 2 kHalo) qp)
    long long img_adj;  // complex elements per adjoint image (P*P)
    float tn;           // (float)(2n)
    float inv2n;        // 1/(2n)
    float wexp;         // pi^2/mu
    float cw;           // (pi/mu)/n : gather weight scale and 1/n of gather
    int T;              // tile core side
    int NT;             // tiles per side P/T
    // launch shapes chosen per problem (tunable): slices per block of the
    // tensor-core gather (1..64), and blocks of the persistent tensor-core
    // scatter (0: one per SM)
    int zper;
    int sc_grid;
};

// Weights of one polar sample restricted to one 16x16 tile of the adjoint
// plan (zero outside the sample's 9x9 stencil), with its ray and the mask of
// tile rows its stencil covers (thm = theta << 16 | mask, theta < 65536),
// its detector index and row factor (-1)^(k+1) shiftadj(k) (pi/mu)/n.
struct AdjRec {
    float wx[16];
    float wy[16];
    int thm;
    int k;
    float2 sf;
};

// Per-angle constants uploaded at geometry set-up.
struct GeoDev {
    float2 *sincos = nullptr;    // [ntheta] (sin, cos) of theta
    float2 *kmat = nullptr;      // [ntheta][m]  K'(theta,j) = ntheta/sqrt(m) sum_i phi_i(theta) conj(phi_i(t_j))
    float2 *shiftfwd = nullptr;  // [n]
    float2 *shiftadj = nullptr;  // [n]
    float *deapod = nullptr;     // [n] exp(mu (x-n/2)^2)
    uint32_t *fwd_pts = nullptr; // point ids theta*n+k sorted by tile
    int4 *fwd_items = nullptr;   // (tile, start, count, 0): direct gather (k_gather_fwd)
    int n_fwd_items = 0;
    int4 *fwd_tc_items = nullptr; // (tile, start, count, rays): tensor-core gather (k_gather_tc)
    int n_fwd_tc_items = 0;
    uint32_t *adj_pts = nullptr; // point ids, one entry per tile a stencil touches
    int4 *adj_items = nullptr;   // (tile, start, count, split)
    int n_adj_items = 0;
    int *split_tiles = nullptr;  // tiles with more than one adjoint item
    int n_split_tiles = 0;
    int *err = nullptr;          // device counter of host/device bin disagreements
    bool tc_scatter = false;     // adjoint time-sample mixing on the tensor cores (k_scatter_tc)
    AdjRec *adj_recs = nullptr;  // geometry records of adj_pts (tensor-core scatter only)
    int n_adj_busy = 0;          // leading adj_items with samples (items are sorted by count)
    // tensor-core scatter tables: each busy item's entries in runs of whole
    // rays (at most one MMA batch of rays and scatter_tc_table_capacity()
    // entries); item i owns tables [adj_tab_base[i],
    // adj_tab_base[i+1]); adj_tabs = (first entry, count, segmentation offset
    // and size in 32-bit words); adj_info = the tables' ray segmentation
    int4 *adj_tabs = nullptr;
    int *adj_tab_base = nullptr;
    uint32_t *adj_info = nullptr;
    int n_adj_tabs = 0;
    // direction path (dir_kernels.cu, DirPlan): sincos then holds one
    // (sin, cos) per direction, adj_pts / adj_items / adj_recs / adj_tabs the
    // direction positions' adjoint entries (ray index := direction index)
    bool dirs = false;
    int ndir = 0;
    int *dray_start = nullptr;    // [ndir + 1]
    uint32_t *drays = nullptr;    // theta | opposite << 31
    float *dtau = nullptr;        // per ray: offset across the direction (DirPlan::tau)
    float4 *demix = nullptr;      // adjoint E, E_perp per (slice, position): dir_mix_bytes(demix_slices, ndir, n)
    int demix_slices = 0;
    uint32_t *dfwd_pos = nullptr; // positions d*n + q sorted by origin tile
    int4 *dfwd_items = nullptr;   // (tile, start, count, 0)
    int n_dfwd_items = 0;
};

// Host-side angle plan (built in plan.cpp).
struct HostPlan {
    std::vector<float2> sincos;
    std::vector<uint32_t> fwd_pts;
    std::vector<int4> fwd_items;
    std::vector<int4> fwd_tc_items;
    std::vector<uint32_t> adj_pts;
    std::vector<int4> adj_items;
    std::vector<int> split_tiles;
};

// Forward work items hold whole rays of one tile and at most fwd_cap samples;
// an item with at least tc_min_spr samples per ray goes to the tensor-core
// gather (tc_min_spr < 0: none does).
HostPlan build_plan(const float *theta, int n, int ntheta, int T, int fwd_cap, int adj_cap, float tc_min_spr);

// Rays grouped by direction (theta modulo pi), for scans that revisit their
// angles over several half-turns: the rays of one direction sample the same
// positions, so the USFFT interpolates once per position (dir_kernels.cu).
struct DirPlan {
    int ndir = 0;
    std::vector<float2> sincos;     // [ndir] (sin, cos) of each direction's representative ray
    std::vector<int> ray_start;     // [ndir + 1]: rays of direction d are rays[ray_start[d] .. ray_start[d+1])
    std::vector<uint32_t> rays;     // theta index | opposite << 31 (sample k of an opposite ray is position n - k)
    std::vector<float> tau;         // per ray (order of rays): its samples' offset across the direction, in
                                    // grid cells per unit of (q - n/2)/n
    std::vector<uint32_t> fwd_pos;  // positions d*n + q (1 <= q < n) sorted by the tile of the stencil origin
    std::vector<int4> fwd_items;    // (tile, start, count, 0): at most fwd_cap positions of one tile
    std::vector<uint32_t> adj_pos;  // one entry per tile a position's stencil touches
    std::vector<int4> adj_items;    // (tile, start, count, 0), one per tile, busiest first
};
// Defaults of the direction path: rays are grouped when their samples agree
// within kDirTolCells grid cells, and the path is taken when the rays average
// at least kDirMinGroup per direction.
constexpr double kDirTolCells = 2e-3;
constexpr double kDirMinGroup = 2.5;
// Groups rays whose sample positions agree within tol_cells grid cells.
// Returns false (plan unused) when the rays average fewer than min_group per
// direction or there are 65536 directions or more.
bool build_dir_plan(const float *theta, int n, int ntheta, int T, int fwd_cap, double tol_cells, double min_group,
                    DirPlan &dp);

// 32-bit words of an adjoint table's ray segmentation with nseg rays: [0]
// nseg, [4 + 8 s + w] the table rows [lo, hi) of ray s that cover rows 2w,
// 2w+1 of the tile (lo | hi << 16), then the first row of every ray and the
// table size as 16-bit values; padded to 16 bytes.
__host__ __device__ constexpr int adj_info_words(int nseg) { return (4 + 8 * nseg + (nseg + 2) / 2 + 3) & ~3; }
// The direction path's form: [4 + 16 s + b] the rows [lo, hi) of direction s
// whose stencils touch 4x4-cell block b of the tile (rows 4 (b >> 2) .. + 3,
// columns 4 (b & 3) .. + 3).
__host__ __device__ constexpr int dir_adj_info_words(int nseg) {
    return (4 + 16 * nseg + (nseg + 2) / 2 + 3) & ~3;
}

// ---- USFFT kernel launchers (usfft_kernels.cu) ----
void launch_deapod_pad(const float *u, float *spec, int nimg, const float *deapod, const UsGeo &g,
                       cudaStream_t s);
// fill the halo of nimg forward spectra after the R2C transform
void launch_spec_halo(float2 *spec, int nimg, const UsGeo &g, cudaStream_t s);
void launch_gather_fwd(const float2 *spec, float2 *rows, int zb, const GeoDev &gd, const UsGeo &g,
                       const CUtensorMap *tmap, cudaStream_t s);
void launch_finish_fwd(const float2 *rows, const float *gdata, float *out, int zb, float tau,
                       int residual, const UsGeo &g, cudaStream_t s);
void launch_adj_prep(const float *h, float *rowsr, int zb, const UsGeo &g, cudaStream_t s);
void launch_zero_split(float2 *spec, int zb, const GeoDev &gd, const UsGeo &g, cudaStream_t s);
void launch_scatter_adj(const float2 *rowsc, float2 *spec, int zb, const GeoDev &gd,
                        const UsGeo &g, cudaStream_t s);
void launch_crop_accum(const float2 *spec, float *u, int zb, float tau, const float *deapod,
                       const UsGeo &g, cudaStream_t s);
// the same from the real output of the C2R inverse (rows of 2 (P/2+1) floats)
void launch_crop_accum_real(const float *out, float *u, int zb, float tau, const float *deapod, const UsGeo &g,
                            cudaStream_t s);
// tensor-core gather (gather_tc.cu): items of fwd_tc_items, time samples
// [jbase, jbase + 16)
void launch_gather_tc(float2 *rows, int zb, const GeoDev &gd, const UsGeo &g, const CUtensorMap &tmap, int jbase,
                      int accumulate, cudaStream_t s);
// TMA descriptor of the forward spectra of a batch (zb*m images), boxes of
// 16 images x 24 rows x 26 cells
void make_spec_tensor_map(CUtensorMap *map, float2 *spec, int nimg, const UsGeo &g);
void gather_tc_prepare();
// tensor-core scatter (scatter_tc.cu): all adjoint items, time samples [jbase, jbase + 16),
// added into the zeroed Hermitian half planes [z][t][P][P/2+1] of the C2R inverse
void launch_scatter_tc(const float2 *rowsc, float2 *spec, int zb, const GeoDev &gd, const UsGeo &g, int jbase,
                       cudaStream_t s);
void scatter_tc_prepare();
void launch_adj_records(AdjRec *recs, const GeoDev &gd, const UsGeo &g, cudaStream_t s);
// entries per scatter table, and the 32-bit words of a table's segmentation
// with nseg rays (count, per-warp sample ranges, ray starts)
int scatter_tc_table_capacity();
int scatter_tc_batch_rays();  // rays per tensor-core batch
int scatter_tc_info_words(int nseg);
// fill adj_info from the records (after launch_adj_records)
void launch_adj_tabinfo(const GeoDev &gd, cudaStream_t s);
// direction path (dir_kernels.cu): forward rows of all rays from the
// positions' interpolated spectra (time samples [jbase, jbase + 16),
// accumulated into rows when accumulate != 0), and the adjoint scatter into
// the zeroed Hermitian half planes (as launch_scatter_tc)
void launch_gather_dir(float2 *rows, const float2 *spec, int zb, const GeoDev &gd, const UsGeo &g, int jbase,
                       int accumulate, cudaStream_t s);
void launch_scatter_dir(const float2 *rowsc, float2 *spec, int zb, const GeoDev &gd, const UsGeo &g, int jbase,
                        cudaStream_t s);
// geometry records of the direction path's adjoint entries (as
// launch_adj_records, with sf = (A, Bx), k = float bits of By: the first-order
// weight of entry p at tile cell (cx, cy) is w (A + B . (cx, cy)),
// B = c1/(2n) (cos, -sin) of the direction, c1 = 2 pi^2/mu / (2n))
void launch_adj_records_dir(AdjRec *recs, const GeoDev &gd, const UsGeo &g, cudaStream_t s);
// their segmentation (dir_adj_info_words per table)
void launch_adj_tabinfo_dir(const GeoDev &gd, cudaStream_t s);
void dir_prepare();           // kernel attributes; once, outside stream capture
int dir_fwd_capacity();       // positions per forward item
int dir_adj_table_capacity(); // entries per adjoint table
int dir_adj_table_dirs();     // directions per adjoint table
size_t dir_mix_bytes(int zb, int ndir, int n);  // the adjoint's per-position mixing buffer
// hand-written 2D FFTs of the zero-padded grids (fft_kernels.cu), P = 2n a
// power of two in [256, 2048]: forward = deapodise/pad/modulate + R2C into
// the halo-padded spectra (halo not filled); inverse = C2R of the Hermitian
// half planes [img][P][hpitch] (overwritten) + crop/deapodise, u += tau * ...
bool pad_fft_supported(int P);
void pad_fft_prepare();
std::vector<float2> pad_fft_twiddles(int P);
// TMA descriptors of the column passes over the spectra buffer (nimg images)
void make_pad_fft_maps(CUtensorMap *fwd, CUtensorMap *inv, float2 *spec, int nimg, const UsGeo &g);
void launch_pad_fft_fwd(const float *u, float2 *spec, int nimg, const float *deapod, const float2 *tw,
                        const CUtensorMap &map, int *err, const UsGeo &g, cudaStream_t s);
void launch_pad_fft_inv_accum(float2 *spec, float *u, int zb, float tau, const float *deapod, const float2 *tw,
                              const CUtensorMap &map, int *err, const UsGeo &g, cudaStream_t s);
// fused residual rows of the inner step (fft_kernels.cu), n a power of two in
// [256, 1024]: gathered rows [z][theta][n] and data g -> the adjoint's row
// spectra [z][theta][n/2+1] (inverse row FFT, residual, fftshift, R2C)
bool resid_rows_supported(int n);
void launch_resid_rows(const float2 *rows, const float *gdata, float2 *out, const float2 *tw_n, int zb,
                       const UsGeo &g, cudaStream_t s);
size_t gather_tc_smem();
int gather_tc_table_capacity();
size_t gather_fwd_smem(const UsGeo &g);
size_t scatter_adj_smem(const UsGeo &g);
void usfft_prepare();  // kernel attributes; call once, outside stream capture
int table_capacity();  // samples per gather work item

// ---- TV / ADMM kernel launchers (tv_kernels.cu) ----
struct TvGeo {
    int n, m, nzp, nchunks;  // chunks processed: nchunks of nzp slices
    long long vol_slab;      // n*n*m
    long long gp;            // grid points per chunk (n+1)^2 (m+1)(nzp+1)
    long long comp_stride;   // elements between SoA components = nchunks_total*gp
    float sg;                // gradient scale 1/(2 cbrt2 lambda1/2)
    float sd;                // divergence scale 1/(4 cbrt2 lambda1/2)
    float lambda1;
};

// u_out = u_in - 0.5 * div(rho (G u_in - psi) + mu) for chunks [c0, c0+nchunks);
// mode 0 reads psi and mu, mode 1 also stores w = mu - rho psi (psi's layout),
// mode 2 reads w only (psi, mu and rho unchanged since the mode-1 step)
void launch_graddiv(const float *u_in, const float *u_old, float *u_out, const float *psi,
                    const float *mu, float *w, int mode, const float *rho, int c0, int nchunks_total,
                    const TvGeo &t, cudaStream_t s);
// shrink + dual update + residual sums into per-block partials
int launch_shrink(const float *u_cur, const float *u_old, float *psi, float *mu, const float *rho,
                  float lambda0, int c0, int nchunks_total, const TvGeo &t, double *partials,
                  cudaStream_t s);
int shrink_blocks(const TvGeo &t, int nchunks);
// sum partials in fixed order, apply the rho rule, append a stats row at *ctr
// (two fixed-order stages; stage1 holds 3*reduce_stage1_parts() doubles)
void launch_reduce_rho(const double *partials, int nparts, double *stage1, float *rho, double *stats, int *ctr,
                       int cap, cudaStream_t s);
int reduce_stage1_parts();
// reference-layout gradient / divergence for the operator API and check_adjoints
// fm points at slab zbase-1 of the extended chunk (zbase = 1 when fm holds
// the two halo slabs, 0 when it holds the chunk only and flgl = flgr = 0)
void launch_gradient_ref(const float *fm, int zbase, float *h2, int flgl, int flgr, const TvGeo &t,
                         cudaStream_t s);
void launch_divergent_ref(float *fn, const float *h2, float tau, const TvGeo &t, cudaStream_t s);
// FP64 dot products: out[0] += sum a*b over count (a==b allowed); deterministic two-pass
void launch_dot(const float *a, const float *b, long long count, double *partials, int nparts,
                double *out, cudaStream_t s);
int dot_parts();

// ---- filtered backprojection helpers (io_kernels.cu) ----
void launch_filter_rows(float2 *rowsc, const float *w, long long nrows, int n, cudaStream_t s);
void launch_fbp_mask(const float *u, float *out, int nslices, int n, int m, float r, cudaStream_t s);

// ---- data ingest (io_kernels.cu) ----
void preprocess(float *out, const void *data, const void *dark, const void *flat, int dtype, int ntheta, int nz,
                int n, int ndark, int nflat);

}  // namespace rectv
