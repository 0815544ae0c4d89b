// Angle plan: polar sample positions binned by tile of the oversampled
// frequency grid.  Built on the host once per geometry (theta is fixed for a
// whole reconstruction, as in rectv::run, src/cuda/rectv.cu:115).
//
// Sample (theta, k), 1 <= k < n, sits at x0 = (k-n/2)/n sin(theta),
// y0 = (k-n/2)/n cos(theta) (takexy, kernels_radonusfft.cuh:66-79); its
// 9x9 Gaussian stencil starts at floor(2n x0) - 4 (gather,
// kernels_radonusfft.cuh:110-119).  k = 0 is never stored: the reference
// zeroes that sample (kernels_radonusfft.cuh:104-108,138-142).
//
// The float arithmetic for x0 and floor(2n x0) is the same sequence of IEEE
// operations the kernels perform, so host bins and device stencils agree.
// This file must be compiled without floating-point contraction.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <exception>
#include <mutex>
#include <thread>
#include <utility>
#include <vector>

#include "rectv_internal.cuh"

namespace rectv {

namespace {
inline int wrapi(int a, int m) {
    a %= m;
    return a < 0 ? a + m : a;
}

// fn(0) .. fn(nthr-1) on nthr host threads (the calling thread runs fn(0))
template <class F>
void parallel_for(int nthr, F &&fn) {
    std::vector<std::thread> pool;
    std::exception_ptr err;
    std::mutex mu;
    for (int w = 1; w < nthr; ++w)
        pool.emplace_back([&, w] {
            try {
                fn(w);
            } catch (...) {
                std::lock_guard<std::mutex> lk(mu);
                if (!err) err = std::current_exception();
            }
        });
    try {
        fn(0);
    } catch (...) {
        std::lock_guard<std::mutex> lk(mu);
        if (!err) err = std::current_exception();
    }
    for (auto &t : pool) t.join();
    if (err) std::rethrow_exception(err);
}
}  // namespace

HostPlan build_plan(const float *theta, int n, int ntheta, int T, int fwd_cap, int adj_cap, float tc_min_spr) {
    HostPlan p;
    const int P = 2 * n;
    const int NT = (P + T - 1) / T;
    const int ntiles = NT * NT;
    p.sincos.resize(ntheta);
    for (int th = 0; th < ntheta; ++th) {
        double t = (double)theta[th];
        p.sincos[th] = make_float2((float)std::sin(t), (float)std::cos(t));
    }
    const long long npts = (long long)ntheta * (n - 1);
    std::vector<int> ftile(npts);
    std::vector<int4> atiles(npts);  // up to 4 tiles, -1 = none
    const float tn = (float)(2 * n);
    std::vector<float> qk(n);
    for (int k = 1; k < n; ++k) qk[k] = (float)(k - n / 2) / (float)n;
    if (T < kTaps) throw Error(1, "tile smaller than the interpolation stencil");
    // Angles are split into contiguous ranges, one per host thread; each
    // thread counts its samples per tile and later places them at its own
    // offsets, so every tile keeps the theta-major sample order.
    const int nthr = std::max(1, std::min<int>((int)std::thread::hardware_concurrency(), std::min(16, ntheta)));
    auto th_range = [&](int w) { return std::make_pair((int)((long long)ntheta * w / nthr),
                                                      (int)((long long)ntheta * (w + 1) / nthr)); };
    std::vector<std::vector<int>> fcw(nthr, std::vector<int>(ntiles, 0)), acw(nthr, std::vector<int>(ntiles, 0));
    auto bin = [&](int w) {
        const auto rg = th_range(w);
        std::vector<int> &fcnt = fcw[w], &acnt = acw[w];
        long long ip = (long long)rg.first * (n - 1);
        for (int th = rg.first; th < rg.second; ++th) {
            const float s = p.sincos[th].x, c = p.sincos[th].y;
            for (int k = 1; k < n; ++k, ++ip) {
                const float q = qk[k];
                float x0 = q * s, y0 = q * c;
                if (x0 >= 0.5f) x0 = 0.5f - 1e-5f;
                if (y0 >= 0.5f) y0 = 0.5f - 1e-5f;
                const int fx = (int)std::floor(tn * x0);
                const int fy = (int)std::floor(tn * y0);
                const int KX = n + fx, KY = n + fy;  // in [0, P)
                const int t = (KY / T) * NT + (KX / T);
                ftile[ip] = t;
                fcnt[t]++;
                // tiles holding any cell of the 9x9 stencil (cells wrap modulo P):
                // a stencil row spans 9 < T cells, so it touches the tiles of its
                // first and last cell and none between
                const int xa = wrapi(KX - kR, P) / T, xb = wrapi(KX + kR, P) / T;
                const int ya = wrapi(KY - kR, P) / T, yb = wrapi(KY + kR, P) / T;
                const int nx = (xa == xb) ? 1 : 2, ny = (ya == yb) ? 1 : 2;
                const int xs[2] = {xa, xb}, ys[2] = {ya, yb};
                int tl[4] = {-1, -1, -1, -1}, nt = 0;
                for (int a = 0; a < ny; ++a)
                    for (int b = 0; b < nx; ++b) tl[nt++] = ys[a] * NT + xs[b];
                atiles[ip] = make_int4(tl[0], tl[1], tl[2], tl[3]);
                for (int i = 0; i < nt; ++i) acnt[tl[i]]++;
            }
        }
    };
    parallel_for(nthr, bin);
    // forward and adjoint: counting sort by tile (stable: theta-major order inside a tile)
    std::vector<long long> foff(ntiles + 1, 0), aoff(ntiles + 1, 0);
    std::vector<int> fcnt(ntiles, 0), acnt(ntiles, 0);
    for (int t = 0; t < ntiles; ++t) {
        for (int w = 0; w < nthr; ++w) {
            fcnt[t] += fcw[w][t];
            acnt[t] += acw[w][t];
        }
        foff[t + 1] = foff[t] + fcnt[t];
        aoff[t + 1] = aoff[t] + acnt[t];
    }
    p.fwd_pts.resize(foff[ntiles]);
    p.adj_pts.resize(aoff[ntiles]);
    {
        // thread w's first slot in tile t: the tile's offset plus the counts of threads before it
        std::vector<std::vector<long long>> fpos(nthr, std::vector<long long>(ntiles)),
            apos(nthr, std::vector<long long>(ntiles));
        for (int t = 0; t < ntiles; ++t) {
            long long f = foff[t], a = aoff[t];
            for (int w = 0; w < nthr; ++w) {
                fpos[w][t] = f;
                apos[w][t] = a;
                f += fcw[w][t];
                a += acw[w][t];
            }
        }
        auto place = [&](int w) {
            const auto rg = th_range(w);
            std::vector<long long> &fp = fpos[w], &ap = apos[w];
            long long ip = (long long)rg.first * (n - 1);
            for (int th = rg.first; th < rg.second; ++th)
                for (int k = 1; k < n; ++k, ++ip) {
                    const uint32_t id = (uint32_t)th * (uint32_t)n + (uint32_t)k;
                    p.fwd_pts[fp[ftile[ip]]++] = id;
                    const int4 a = atiles[ip];
                    const int tl[4] = {a.x, a.y, a.z, a.w};
                    for (int i = 0; i < 4; ++i)
                        if (tl[i] >= 0) p.adj_pts[ap[tl[i]]++] = id;
                }
        };
        parallel_for(nthr, place);
    }
    // forward items: whole rays (runs of equal theta) of one tile, at most
    // fwd_cap samples; rays with several samples each go to the tensor cores
    for (int t = 0; t < ntiles; ++t) {
        long long i = foff[t];
        const long long e = foff[t + 1];
        while (i < e) {
            long long j = i;
            int nrays = 0;
            while (j < e) {
                const uint32_t th = p.fwd_pts[j] / (uint32_t)n;
                long long r = j;
                while (r < e && p.fwd_pts[r] / (uint32_t)n == th) ++r;
                if (r - i > fwd_cap) break;
                j = r;
                ++nrays;
            }
            if (nrays == 0) throw Error(1, "ray longer than a gather work item");
            const int cnt = (int)(j - i);
            if (tc_min_spr >= 0.f && cnt >= tc_min_spr * nrays)
                p.fwd_tc_items.push_back(make_int4(t, (int)i, cnt, nrays));
            else
                p.fwd_items.push_back(make_int4(t, (int)i, cnt, 0));
            i = j;
        }
    }
    for (int t = 0; t < ntiles; ++t) {
        const int c = acnt[t];
        if (c == 0) {
            p.adj_items.push_back(make_int4(t, (int)aoff[t], 0, 0));
            continue;
        }
        const int nit = (c + adj_cap - 1) / adj_cap;
        const int split = nit > 1 ? 1 : 0;
        if (split) p.split_tiles.push_back(t);
        for (int st = 0; st < c; st += adj_cap)
            p.adj_items.push_back(make_int4(t, (int)(aoff[t] + st), std::min(adj_cap, c - st), split));
    }
    // heaviest tiles first, so that they do not finish last
    std::stable_sort(p.adj_items.begin(), p.adj_items.end(),
                     [](const int4 &a, const int4 &b) { return a.z > b.z; });
    return p;
}

// Directions of a scan over several half-turns.  Ray theta samples the line
// through the origin in direction (sin theta, cos theta); sample k sits at
// (k-n/2)/n times that vector, so rays theta and theta + pi (and theta + 2 pi)
// sample the same points: sample k of the opposite ray is sample n-k of the
// other.  Rays whose directions agree within tol_cells / n radians (their
// samples then lie within tol_cells grid cells of each other) share the
// positions of one representative ray, the group member of median angle; a
// ray's own samples lie (q-n/2)/n * tau_r cells across the direction from the
// shared positions (the kernels correct for it to first order).
bool build_dir_plan(const float *theta, int n, int ntheta, int T, int fwd_cap, double tol_cells, double min_group,
                    DirPlan &dp) {
    dp = DirPlan();
    const double pi = 3.14159265358979323846;
    const double tol = tol_cells / (double)n;
    std::vector<double> alpha(ntheta);
    std::vector<float2> sc(ntheta);
    std::vector<uint32_t> opp(ntheta);
    for (int th = 0; th < ntheta; ++th) {
        const double t = (double)theta[th];
        float s = (float)std::sin(t), c = (float)std::cos(t);
        uint32_t o = (s < 0.f || (s == 0.f && c < 0.f)) ? 1u : 0u;
        if (o) {
            s = -s;
            c = -c;
        }
        double a = std::atan2((double)s, (double)c);  // [0, pi]
        if (a > pi - tol) {                           // the same line as a - pi, reversed
            a -= pi;
            s = -s;
            c = -c;
            o ^= 1u;
        }
        alpha[th] = a;
        sc[th] = make_float2(s, c);
        opp[th] = o;
    }
    std::vector<int> order(ntheta);
    for (int i = 0; i < ntheta; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return alpha[a] < alpha[b]; });
    dp.ray_start.push_back(0);
    for (int i = 0; i < ntheta;) {
        int j = i + 1;
        while (j < ntheta && alpha[order[j]] - alpha[order[i]] <= tol) ++j;
        const int med = order[i + (j - i) / 2];  // member of median angle (order is sorted by angle)
        std::sort(order.begin() + i, order.begin() + j);  // rays of a direction in theta order
        dp.sincos.push_back(sc[med]);
        const double sd = sc[med].x, cd = sc[med].y;
        for (int r = i; r < j; ++r) {
            const int th = order[r];
            dp.rays.push_back((uint32_t)th | (opp[th] << 31));
            // offset of the ray's samples across the direction, per unit of
            // (q - n/2)/n, in grid cells: 2n (s_r c_d - c_r s_d) with the
            // ray's exact (orientation-normalised) direction
            const double t = (double)theta[th], sg = opp[th] ? -1.0 : 1.0;
            dp.tau.push_back((float)(2.0 * n * (sg * std::sin(t) * cd - sg * std::cos(t) * sd)));
        }
        dp.ray_start.push_back((int)dp.rays.size());
        i = j;
    }
    dp.ndir = (int)dp.sincos.size();
    if ((double)ntheta < min_group * dp.ndir || dp.ndir >= 65536) return false;

    // positions (d, q), 1 <= q < n: the same float sequence as the kernels
    // (sample_pos), binned by the tile of the stencil origin (forward) and by
    // every tile the stencil touches (adjoint), direction-major inside a tile
    const int P = 2 * n;
    const int NT = (P + T - 1) / T;
    const int ntiles = NT * NT;
    const float tn = (float)(2 * n);
    std::vector<float> qk(n);
    for (int k = 1; k < n; ++k) qk[k] = (float)(k - n / 2) / (float)n;
    const long long npos = (long long)dp.ndir * (n - 1);
    std::vector<int> ftile(npos);
    std::vector<int4> atiles(npos);
    std::vector<long long> fcnt(ntiles + 1, 0), acnt(ntiles + 1, 0);
    long long ip = 0;
    for (int d = 0; d < dp.ndir; ++d) {
        const float s = dp.sincos[d].x, c = dp.sincos[d].y;
        for (int q = 1; q < n; ++q, ++ip) {
            float x0 = qk[q] * s, y0 = qk[q] * c;
            if (x0 >= 0.5f) x0 = 0.5f - 1e-5f;
            if (y0 >= 0.5f) y0 = 0.5f - 1e-5f;
            const int KX = n + (int)std::floor(tn * x0), KY = n + (int)std::floor(tn * y0);
            ftile[ip] = (KY / T) * NT + (KX / T);
            fcnt[ftile[ip]]++;
            const int xa = wrapi(KX - kR, P) / T, xb = wrapi(KX + kR, P) / T;
            const int ya = wrapi(KY - kR, P) / T, yb = wrapi(KY + kR, P) / T;
            const int nx = (xa == xb) ? 1 : 2, ny = (ya == yb) ? 1 : 2;
            const int xs[2] = {xa, xb}, ys[2] = {ya, yb};
            int tl[4] = {-1, -1, -1, -1}, nt = 0;
            for (int a = 0; a < ny; ++a)
                for (int b = 0; b < nx; ++b) tl[nt++] = ys[a] * NT + xs[b];
            atiles[ip] = make_int4(tl[0], tl[1], tl[2], tl[3]);
            for (int i = 0; i < nt; ++i) acnt[tl[i]]++;
        }
    }
    std::vector<long long> foff(ntiles + 1, 0), aoff(ntiles + 1, 0);
    for (int t = 0; t < ntiles; ++t) {
        foff[t + 1] = foff[t] + fcnt[t];
        aoff[t + 1] = aoff[t] + acnt[t];
    }
    dp.fwd_pos.resize(foff[ntiles]);
    dp.adj_pos.resize(aoff[ntiles]);
    {
        std::vector<long long> fp(foff.begin(), foff.end() - 1), ap(aoff.begin(), aoff.end() - 1);
        ip = 0;
        for (int d = 0; d < dp.ndir; ++d)
            for (int q = 1; q < n; ++q, ++ip) {
                const uint32_t id = (uint32_t)d * (uint32_t)n + (uint32_t)q;
                dp.fwd_pos[fp[ftile[ip]]++] = id;
                const int4 a = atiles[ip];
                const int tl[4] = {a.x, a.y, a.z, a.w};
                for (int i = 0; i < 4; ++i)
                    if (tl[i] >= 0) dp.adj_pos[ap[tl[i]]++] = id;
            }
    }
    for (int t = 0; t < ntiles; ++t)
        for (long long i = foff[t]; i < foff[t + 1]; i += fwd_cap)
            dp.fwd_items.push_back(make_int4(t, (int)i, (int)std::min<long long>(fwd_cap, foff[t + 1] - i), 0));
    for (int t = 0; t < ntiles; ++t) dp.adj_items.push_back(make_int4(t, (int)aoff[t], (int)acnt[t], 0));
    // heaviest tiles first (the empty ones last)
    std::stable_sort(dp.adj_items.begin(), dp.adj_items.end(),
                     [](const int4 &a, const int4 &b) { return a.z > b.z; });
    return true;
}

}  // namespace rectv
