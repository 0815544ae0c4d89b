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
#include <vector>

#include "rectv_internal.cuh"

namespace rectv {

namespace {
inline int wrapi(int a, int m) {
    a %= m;
    return a < 0 ? a + m : a;
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
    std::vector<int> fcnt(ntiles, 0), acnt(ntiles, 0);
    const float tn = (float)(2 * n);
    long long ip = 0;
    for (int th = 0; th < ntheta; ++th) {
        const float s = p.sincos[th].x, c = p.sincos[th].y;
        for (int k = 1; k < n; ++k, ++ip) {
            const float q = (float)(k - n / 2) / (float)n;
            float x0 = q * s, y0 = q * c;
            if (x0 >= 0.5f) x0 = 0.5f - 1e-5f;
            if (y0 >= 0.5f) y0 = 0.5f - 1e-5f;
            const int fx = (int)std::floor(tn * x0);
            const int fy = (int)std::floor(tn * y0);
            const int KX = n + fx, KY = n + fy;  // in [0, P)
            const int t = (KY / T) * NT + (KX / T);
            ftile[ip] = t;
            fcnt[t]++;
            // tiles holding any cell of the 9x9 stencil (cells wrap modulo P)
            int xs[kTaps], ys[kTaps], nx = 0, ny = 0;
            for (int i = 0; i < kTaps; ++i) {
                const int tx = wrapi(KX - kR + i, P) / T, ty = wrapi(KY - kR + i, P) / T;
                bool seen = false;
                for (int a = 0; a < nx; ++a) seen |= (xs[a] == tx);
                if (!seen) xs[nx++] = tx;
                seen = false;
                for (int a = 0; a < ny; ++a) seen |= (ys[a] == ty);
                if (!seen) ys[ny++] = ty;
            }
            if (nx > 2 || ny > 2) throw Error(1, "tile smaller than the interpolation stencil");
            int tl[4] = {-1, -1, -1, -1}, nt = 0;
            for (int a = 0; a < ny; ++a)
                for (int b = 0; b < nx; ++b) tl[nt++] = ys[a] * NT + xs[b];
            atiles[ip] = make_int4(tl[0], tl[1], tl[2], tl[3]);
            for (int i = 0; i < nt; ++i) acnt[tl[i]]++;
        }
    }
    // forward: counting sort by tile (stable: theta-major order inside a tile)
    std::vector<long long> foff(ntiles + 1, 0), aoff(ntiles + 1, 0);
    for (int t = 0; t < ntiles; ++t) {
        foff[t + 1] = foff[t] + fcnt[t];
        aoff[t + 1] = aoff[t] + acnt[t];
    }
    p.fwd_pts.resize(foff[ntiles]);
    p.adj_pts.resize(aoff[ntiles]);
    {
        std::vector<long long> fpos(foff.begin(), foff.end() - 1), apos(aoff.begin(), aoff.end() - 1);
        ip = 0;
        for (int th = 0; th < ntheta; ++th)
            for (int k = 1; k < n; ++k, ++ip) {
                const uint32_t id = (uint32_t)th * (uint32_t)n + (uint32_t)k;
                p.fwd_pts[fpos[ftile[ip]]++] = id;
                const int4 a = atiles[ip];
                const int tl[4] = {a.x, a.y, a.z, a.w};
                for (int i = 0; i < 4; ++i)
                    if (tl[i] >= 0) p.adj_pts[apos[tl[i]]++] = id;
            }
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

}  // namespace rectv
