// tables.cpp -- host FP64 tables of the NUDIM engine.  Compiled with
// -ffp-contract=off so that x86-64 and aarch64 hosts build identical tables.
#include "tables.h"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <thread>

namespace nudim {

static constexpr int kM = 6;
static constexpr int kW = 2 * kM + 2;

// fn(begin, end, part) over [0, n) split into contiguous parts, one host
// thread each (at most 16; one part for small n).  Parts are ordered:
// part k covers indices below those of part k + 1.
template <typename F> static int parallel_for(int n, int grain, F &&fn)
{
    int hw = (int)std::thread::hardware_concurrency();
    int nt = std::max(1, std::min({16, hw > 0 ? hw : 1, n / std::max(1, grain)}));
    if (nt == 1) {
        fn(0, n, 0);
        return 1;
    }
    std::vector<std::thread> th;
    for (int k = 0; k < nt; k++)
        th.emplace_back([&, k] { fn((int)((long)n * k / nt), (int)((long)n * (k + 1) / nt), k); });
    for (auto &x : th) x.join();
    return nt;
}

int grid_size(int N)
{
    int p = 1;
    while (p < N) p <<= 1;
    return 2 * p;
}

int equal_angle_count(double amin, double amax, double ainterval)
{
    return (int)((amax - amin) / ainterval + 0.5) + 1;
}

// Radius by repeated addition of 1/nx starting at -1/2 - 1/nx, node
// (r sin g, r cos g) with g in degrees and the truncated pi of grid.h.
void equal_angle_sample_2d(double amin, double amax, double ainterval, int nx, double *x)
{
    int ns = equal_angle_count(amin, amax, ainterval);
    double angle = amin - ainterval;
    for (int s = 0; s < ns; s++) {
        angle += ainterval;
        double step = 1.0 / nx, r = -0.5 - step;
        double sg = sin(angle / 180 * kRefPi), cg = cos(angle / 180 * kRefPi);
        double *xs = x + (size_t)s * nx * 2;
        for (int i = 0; i < nx; i++) {
            r += step;
            xs[2 * i + 0] = r * sg;
            xs[2 * i + 1] = r * cg;
        }
    }
}

void polar_factors(double amin, double amax, double ainterval, int nx, double *r, double *sg,
                   double *cg)
{
    // the same loops and operations as equal_angle_sample_2d: node (a, i) is
    // (r[i] sg[a], r[i] cg[a]) up to the one rounding of the product
    int ns = equal_angle_count(amin, amax, ainterval);
    double angle = amin - ainterval;
    for (int s = 0; s < ns; s++) {
        angle += ainterval;
        sg[s] = sin(angle / 180 * kRefPi);
        cg[s] = cos(angle / 180 * kRefPi);
    }
    double step = 1.0 / nx, rr = -0.5 - step;
    for (int i = 0; i < nx; i++) {
        rr += step;
        r[i] = rr;
    }
}

void uniform_sample_2d(int nx, int nz, double *x)
{
    double ix = 1.0 / nx, iz = 1.0 / nz, z0 = -0.5 - iz;
    for (int j = 0; j < nz; j++) {
        z0 += iz;
        double x0 = -0.5 - ix;
        for (int i = 0; i < nx; i++) {
            x0 += ix;
            x[2 * ((size_t)j * nx + i) + 0] = x0;
            x[2 * ((size_t)j * nx + i) + 1] = z0;
        }
    }
}

int polar_lines(double gam_min, double interval, double padangle, double *pad_min,
                double *pad_max)
{
    int ntmp = (int)((-90 - gam_min) / interval);
    double lo = gam_min + ntmp * interval;
    ntmp = (int)((90 - gam_min) / interval);
    double hi = gam_min + ntmp * interval;
    if (pad_min) *pad_min = lo;
    if (pad_max) *pad_max = hi;
    return equal_angle_count(lo, hi, padangle);
}

// Modified Bessel I0 by its power series (positive terms; accurate to a few
// ulp for the arguments m*b < 40 used here).
static double bessel_i0(double x)
{
    double q = 0.25 * x * x, term = 1.0, sum = 1.0;
    for (int k = 1; k < 500; k++) {
        term *= q / ((double)k * (double)k);
        sum += term;
        if (term < sum * 1e-18) break;
    }
    return sum;
}

// Kaiser-Bessel window of the published NFFT method at distance dn (grid
// cells) from the node: sinh(b*sqrt(m^2-dn^2)) / (pi*sqrt(m^2-dn^2)),
// continued analytically (sin branch) beyond the cut-off.
static double kb_phi(double dn, double b)
{
    double a = (double)kM * kM - dn * dn;
    if (a > 0) {
        double s = sqrt(a);
        return sinh(b * s) / (kTruePi * s);
    }
    if (a < 0) {
        double s = sqrt(-a);
        return sin(b * s) / (kTruePi * s);
    }
    return b / kTruePi;
}

// n * phi_hat(k) = I0(m * sqrt(b^2 - (2 pi k / n)^2)).
static double kb_phi_hat(int k, int n, double b)
{
    double t = 2.0 * kTruePi * (double)k / (double)n;
    return bessel_i0((double)kM * sqrt(b * b - t * t));
}

int build_nfft_tables(int N0, int N1, int M, const double *x, int ty, int tx, NfftTables *t)
{
    if (N0 <= 0 || N1 <= 0 || M < 0 || (N0 & 1) || (N1 & 1)) return -1;
    t->N0 = N0;
    t->N1 = N1;
    t->M = M;
    t->n0 = grid_size(N0);
    t->n1 = grid_size(N1);
    double b0 = kTruePi * (2.0 - 1.0 / ((double)t->n0 / (double)N0));
    double b1 = kTruePi * (2.0 - 1.0 / ((double)t->n1 / (double)N1));
    t->u0.assign(M, 0);
    t->u1.assign(M, 0);
    t->psi.assign((size_t)M * 2 * kW, 0.0);
    // A node whose coordinate equals that of an earlier node of the same
    // part (the previous node, or the node `per` earlier: a uniform grid's
    // rows repeat both) copies its window values instead of evaluating the
    // Kaiser-Bessel function again; the values are the same either way.
    int per = 0;
    for (int j = 1; j < M && j < 65536; j++)
        if (x[2 * (size_t)j] == x[0]) {
            per = j;
            break;
        }
    parallel_for(M, 2048, [&](int j0, int j1, int) {
        for (int j = j0; j < j1; j++) {
            for (int d = 0; d < 2; d++) {
                int n = d ? t->n1 : t->n0;
                double b = d ? b1 : b0;
                const double xv = x[2 * (size_t)j + d];
                double xn = xv * (double)n;
                int u = (int)floor(xn) - kM;
                (d ? t->u1 : t->u0)[j] = u;
                double *ps = t->psi.data() + (size_t)j * 2 * kW + (size_t)d * kW;
                int src = -1;
                if (j > j0 && x[2 * (size_t)(j - 1) + d] == xv) src = j - 1;
                else if (per && j - per >= j0 && x[2 * (size_t)(j - per) + d] == xv) src = j - per;
                if (src >= 0) {
                    const double *q = t->psi.data() + (size_t)src * 2 * kW + (size_t)d * kW;
                    for (int s = 0; s < kW; s++) ps[s] = q[s];
                } else {
                    for (int s = 0; s < kW; s++) ps[s] = kb_phi(xn - (double)(u + s), b);
                }
            }
        }
    });
    t->c0.resize(N0);
    t->c1.resize(N1);
    for (int k = 0; k < N0; k++) t->c0[k] = 1.0 / kb_phi_hat(k - N0 / 2, t->n0, b0);
    for (int k = 0; k < N1; k++) t->c1[k] = 1.0 / kb_phi_hat(k - N1 / 2, t->n1, b1);

    t->ty = std::min(ty, t->n0);
    t->tx = std::min(tx, t->n1);
    t->nty = t->n0 / t->ty;
    t->ntx = t->n1 / t->tx;
    return 0;
}

void build_tile_lists(const NfftTables &t, std::vector<int> *off, std::vector<int> *nodes)
{
    const int M = t.M;
    int ntiles = t.nty * t.ntx;
    std::vector<int> cnt(ntiles + 1, 0);
    auto visit = [&](int j, auto &&fn) {
        int rows[16], cols[16], nr = 0, nc = 0;
        for (int s = 0; s < kW; s++) {
            int r = ((t.u0[j] + s) & (t.n0 - 1)) / t.ty;
            int c = ((t.u1[j] + s) & (t.n1 - 1)) / t.tx;
            bool hr = false, hc = false;
            for (int q = 0; q < nr; q++) hr |= rows[q] == r;
            for (int q = 0; q < nc; q++) hc |= cols[q] == c;
            if (!hr && nr < 16) rows[nr++] = r;
            if (!hc && nc < 16) cols[nc++] = c;
        }
        for (int a = 0; a < nr; a++)
            for (int c = 0; c < nc; c++) fn(rows[a] * t.ntx + cols[c]);
    };
    for (int j = 0; j < M; j++) visit(j, [&](int tile) { cnt[tile + 1]++; });
    for (int i = 0; i < ntiles; i++) cnt[i + 1] += cnt[i];
    *off = cnt;
    nodes->assign(cnt[ntiles], 0);
    std::vector<int> pos(cnt.begin(), cnt.end() - 1);
    for (int j = 0; j < M; j++) visit(j, [&](int tile) { (*nodes)[pos[tile]++] = j; });
}

void cgnr_weights(int A, int np, double padangle, double *w)
{
    double h = (double)(np / 2);
    for (int a = 0; a < A; a++)
        for (int i = 0; i < np; i++) {
            if (i == np / 2)
                w[(size_t)a * np + i] = kRefPi / (4 * A * (h * h));
            else
                w[(size_t)a * np + i] = padangle / 180 * kRefPi * abs(i - np / 2) / (h * h);
        }
}

void classify_lines(double pad_min, double padangle, double gam_min, double gam_max,
                    double interval, int A, std::vector<int> *known, std::vector<int> *order)
{
    known->assign(A, 0);
    order->assign(A, 0);
    for (int a = 0; a < A; a++) {
        double angle = pad_min + a * padangle;
        int span = (int)(interval / padangle + 0.5);
        int seq = (int)((angle - gam_min) / padangle + 0.5);
        if ((angle < gam_min) || (angle > gam_max) || (seq % span != 0)) continue;
        if (abs((int)angle) < 1e-5) continue;  // cross-validation band (-1, 1)
        (*known)[a] = 1;
        (*order)[a] = (int)((angle - gam_min) / interval + 0.5);
    }
}

void mt19937_uniform(uint32_t seed, size_t n, double *out)
{
    uint32_t mt[624];
    int mti;
    mt[0] = seed == 0 ? 4357u : seed;
    for (mti = 1; mti < 624; mti++)
        mt[mti] = 1812433253u * (mt[mti - 1] ^ (mt[mti - 1] >> 30)) + (uint32_t)mti;
    for (size_t q = 0; q < n; q++) {
        if (mti >= 624) {
            for (int k = 0; k < 624; k++) {
                uint32_t y = (mt[k] & 0x80000000u) | (mt[(k + 1) % 624] & 0x7fffffffu);
                mt[k] = mt[(k + 397) % 624] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
            }
            mti = 0;
        }
        uint32_t y = mt[mti++];
        y ^= y >> 11;
        y ^= (y << 7) & 0x9d2c5680u;
        y ^= (y << 15) & 0xefc60000u;
        y ^= y >> 18;
        out[q] = (double)y / 4294967296.0;
    }
}

}  // namespace nudim

namespace nudim {

void fft_twiddles(int n, std::vector<double> *tw)
{
    tw->resize(2 * (size_t)n);
    for (int k = 0; k < n; k++) {
        double a = 2.0 * kTruePi * (double)k / (double)n;
        (*tw)[2 * k] = cos(a);
        (*tw)[2 * k + 1] = -sin(a);
    }
}

template <typename Wt>
int build_fused_lists(const NfftTables &t, int BC, int BCa, bool pair_rows, FusedLists<Wt> *L,
                      bool adjoint)
{
    const int kWin = 2 * 6 + 2;
    if (BC <= 0 || t.n1 % BC) return -1;
    if (BCa <= 0 || BCa > 32 || 32 % BCa || t.n1 % BCa) return -1;
    int n0 = t.n0, n1 = t.n1, M = t.M;
    int R = 32 / BCa;
    if (n0 % R) return -1;
    L->BC = BC;
    L->BCa = BCa;
    L->R = R;
    L->nblk = n1 / BC;
    L->nblka = n1 / BCa;
    L->nbands = n0 / R;
    int nblk = L->nblk, nb = L->nbands;
    // ---- trafo lists: blocks met by each node's 14 window columns
    std::vector<std::vector<int>> per(nblk);
    L->nslots.assign(M, 0);
    L->smax = 0;
    // a window may not meet the same block twice (possible only when
    // n1 < 13 + BC): the column pass sums a node's whole block at once
    if (n1 < kWin - 1 + BC && nblk > 1) return -2;
    for (int j = 0; j < M; j++) {
        int slot = 0, last = -1;
        for (int s = 0; s < kWin; s++) {
            int b = ((t.u1[j] + s) & (n1 - 1)) / BC;
            if (b == last) continue;
            per[b].push_back(j * 8 + slot);
            slot++;
            last = b;
        }
        L->nslots[j] = (unsigned char)slot;
        if (slot > L->smax) L->smax = slot;
    }
    if (L->smax > 8) return -1;
    // Entry order inside a block (one column-pass lane per entry): entries
    // with equal numbers of window columns inside the block side by side
    // (longest first), so a warp's lanes run equal loops; inside such a run
    // the first window rows u0 cycle through the residues mod 16, so the
    // lanes of a warp read shared-memory rows spread over all banks.  The
    // column pass reads rows in aligned pairs (pair_rows, 8-byte complex) or
    // singly (16-byte complex); the residue order puts 8 distinct 16-byte
    // slots of a 128-byte line in every 8 consecutive lanes.
    static const int kOrderPairs[16] = {0, 2, 4, 6, 8, 10, 12, 14, 1, 3, 5, 7, 9, 11, 13, 15};
    parallel_for(nblk, 1, [&](int b0, int b1, int) {
    for (int b = b0; b < b1; b++) {
        auto cols = [&](int en) {
            int j = en / 8, k = 0;
            for (int s = 0; s < kWin; s++) k += ((t.u1[j] + s) & (n1 - 1)) / BC == b;
            return k;
        };
        std::vector<std::pair<int, int>> key(per[b].size());
        for (size_t i = 0; i < key.size(); i++) key[i] = {-cols(per[b][i]), per[b][i]};
        std::sort(key.begin(), key.end());
        std::vector<int> out;
        out.reserve(key.size());
        for (size_t i = 0; i < key.size();) {
            size_t k = i;
            while (k < key.size() && key[k].first == key[i].first) k++;
            std::vector<int> bucket[16];
            for (size_t q = i; q < k; q++)
                bucket[t.u0[key[q].second / 8] & 15].push_back(key[q].second);
            size_t head[16] = {0};
            for (size_t left = k - i; left > 0;)
                for (int q = 0; q < 16; q++) {
                    int r = pair_rows ? kOrderPairs[q] : q;
                    if (head[r] < bucket[r].size()) {
                        out.push_back(bucket[r][head[r]++]);
                        left--;
                    }
                }
            i = k;
        }
        per[b] = out;
    }
    });
    L->blk_off.assign(nblk + 1, 0);
    for (int b = 0; b < nblk; b++) L->blk_off[b + 1] = L->blk_off[b] + (int)per[b].size();
    L->ent.clear();
    L->ent.reserve(L->blk_off[nblk]);
    for (int b = 0; b < nblk; b++) L->ent.insert(L->ent.end(), per[b].begin(), per[b].end());
    // per entry, structure of arrays over the nE entries: the even first row
    // rb of the window, the block columns it covers (first cl0, count cnt;
    // column q is (cl0 + q) mod BC), 16 row weights aligned to rb (zero
    // outside the window) and the cnt column weights.
    const size_t nE = L->ent.size();
    L->nq = nblk > 1 ? std::min(BC, kWin) : kWin;
    L->ent_rb.assign(nE, 0);
    L->ent_cc.assign(nE, 0);
    L->ent_qa.alloc(16 * nE);
    L->ent_q1.alloc((size_t)L->nq * nE);
    Wt *qa = L->ent_qa.data(), *q1 = L->ent_q1.data();
    const int nq = L->nq;
    parallel_for(nblk, 1, [&](int b0, int b1, int) {
    for (int b = b0; b < b1; b++)
        for (int e = L->blk_off[b]; e < L->blk_off[b + 1]; e++) {
            int j = L->ent[e] / 8, ux = t.u0[j], uy = t.u1[j], col0 = b * BC;
            int t1lo = 0, cl0 = uy & (n1 - 1), cnt = kWin;
            if (nblk > 1) {
                int d = (col0 - uy) & (n1 - 1);
                cl0 = 0;
                if (d < kWin) t1lo = d;
                else cl0 = (uy - col0) & (n1 - 1);
                cnt = std::min(kWin - t1lo, BC - cl0);
            }
            const double *ps = &t.psi[(size_t)j * 2 * kWin];
            int odd = ux & 1;
            L->ent_rb[e] = ux - odd;
            L->ent_cc[e] = cl0 | (cnt << 8) | (odd << 16);
            for (int i = 0; i < 16; i++) {
                int t0 = i - odd;
                qa[(size_t)i * nE + e] = (Wt)(t0 >= 0 && t0 < kWin ? ps[t0] : 0.0);
            }
            for (int q = 0; q < nq; q++)
                q1[(size_t)q * nE + e] = (Wt)(q < cnt ? ps[kWin + t1lo + q] : 0.0);
        }
    });
    // ---- adjoint lists: tiles of R x BCa grid points (one per warp lane);
    // per tile the nodes whose window meets it, ascending.  Tiles are
    // numbered block-major: tile = b * nbands + v.
    if (!adjoint) {
        L->band_off.assign(1, 0);
        L->band_node.assign(1, 0);
        L->band_w.alloc(0);
        L->band_ord.clear();
        return 0;
    }
    const int nblka = L->nblka;
    // the blocks and bands met by node j's window (each once)
    auto visit = [&](int j, std::vector<int> &bstamp, std::vector<int> &vstamp, auto &&fn) {
        int blks[16], bands[16], nbk = 0, nbd = 0;
        for (int s = 0; s < kWin; s++) {
            int b = ((t.u1[j] + s) & (n1 - 1)) / BCa;
            int v = ((t.u0[j] + s) & (n0 - 1)) / R;
            if (bstamp[b] != j) {
                bstamp[b] = j;
                blks[nbk++] = b;
            }
            if (vstamp[v] != j) {
                vstamp[v] = j;
                bands[nbd++] = v;
            }
        }
        for (int a = 0; a < nbk; a++)
            for (int c = 0; c < nbd; c++) fn((size_t)blks[a] * nb + bands[c]);
    };
    size_t ntiles = (size_t)nblka * nb;
    // counts per (node range, tile), node ranges in ascending order; a
    // tile's entries of range k follow those of range k - 1, so every list
    // stays in ascending node order
    const int kParts = 16;
    std::vector<std::vector<int>> pc(kParts);
    int nparts = parallel_for(M, 4096, [&](int j0, int j1, int k) {
        std::vector<int> bs(nblka, -1), vs(nb, -1);
        pc[k].assign(ntiles, 0);
        for (int j = j0; j < j1; j++) visit(j, bs, vs, [&](size_t tile) { pc[k][tile]++; });
    });
    std::vector<int> cnt(ntiles + 1, 0);
    for (size_t i = 0; i < ntiles; i++) {
        int sum = 0;
        for (int k = 0; k < nparts; k++) sum += pc[k][i];
        cnt[i + 1] = cnt[i] + sum;
    }
    L->band_off = cnt;
    L->band_node.assign(cnt[ntiles], 0);
    // per entry the tile's window weights: R row weights psi0(v*R + rr - u0)
    // then BCa column weights psi1(b*BCa + cc - u1), zero outside the window
    const int W = R + BCa;
    L->band_w.alloc((size_t)cnt[ntiles] * W);
    parallel_for(M, 4096, [&](int j0, int j1, int k) {
        // first slot of this node range in every tile
        std::vector<int> pos(ntiles);
        for (size_t i = 0; i < ntiles; i++) {
            int off = cnt[i];
            for (int q = 0; q < k; q++) off += pc[q][i];
            pos[i] = off;
        }
        std::vector<int> bs(nblka, -1), vs(nb, -1);
        for (int j = j0; j < j1; j++)
            visit(j, bs, vs, [&](size_t tile) {
                int e = pos[tile]++;
                L->band_node[e] = j;
                int b = (int)(tile / nb), v = (int)(tile % nb);
                Wt *w = L->band_w.data() + (size_t)e * W;
                const double *ps = &t.psi[(size_t)j * 2 * kWin];
                for (int rr = 0; rr < R; rr++) {
                    int d = (v * R + rr - t.u0[j]) & (n0 - 1);
                    w[rr] = (Wt)(d < kWin ? ps[d] : 0.0);
                }
                for (int cc = 0; cc < BCa; cc++) {
                    int d = (b * BCa + cc - t.u1[j]) & (n1 - 1);
                    w[R + cc] = (Wt)(d < kWin ? ps[kWin + d] : 0.0);
                }
            });
    });
    // every tile once, longest list first (ties by tile number): the
    // spreading gather hands them out in this order
    L->band_ord.resize(ntiles);
    for (size_t i = 0; i < ntiles; i++) L->band_ord[i] = (int)i;
    std::stable_sort(L->band_ord.begin(), L->band_ord.end(), [&](int x, int y) {
        return cnt[(size_t)x + 1] - cnt[x] > cnt[(size_t)y + 1] - cnt[y];
    });
    return 0;
}

template int build_fused_lists<float>(const NfftTables &, int, int, bool, FusedLists<float> *,
                                      bool);
template int build_fused_lists<double>(const NfftTables &, int, int, bool, FusedLists<double> *,
                                       bool);

}  // namespace nudim
