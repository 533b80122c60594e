"""The fused NFFT's host-built work lists (nudim_gb300/csrc/tables.cpp:
build_fused_lists) on the CPU: every node's trafo entries (per column block)
and adjoint tile entries (per R x BCa tile) must reproduce exactly its window
weights psi0[r - u0] * psi1[c - u1] on its 14 x 14 window of the oversampled
grid (wrapping at the edges), each grid point once; tile lists are in
ascending node order, every tile listed once, longest list first; a
node's trafo entries share its first row and row weights.  The grid
path's spreading tile lists (build_tile_lists) hold, per tile, exactly the
nodes whose window meets it, ascending.  A g++ harness links tables.cpp
directly (no GPU)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "nudim_gb300", "csrc")

HARNESS = r"""
#include "tables.h"
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <random>
#include <vector>
using namespace nudim;
static const int kWin = 14;

template <typename W>
static int check(int N, int M, int BC, bool pair_rows, unsigned seed)
{
    std::mt19937 g(seed);
    std::uniform_real_distribution<double> U(-0.5, 0.5);
    std::vector<double> x(2 * (size_t)M);
    for (auto &v : x) v = U(g);
    x[0] = -0.5; x[1] = -0.5;                 // windows that wrap on both axes
    x[2] = 0.5 - 1e-9; x[3] = 0.5 - 1e-9;
    NfftTables t;
    if (build_nfft_tables(N, N, M, x.data(), 16, 16, &t)) return 10;
    FusedLists<W> L;
    int rc = build_fused_lists<W>(t, BC, 4, pair_rows, &L);
    if (rc) return 20 + (-rc);
    const int n0 = t.n0, n1 = t.n1;
    // expected dense weights per node, as the lists store them (W precision)
    auto expect = [&](int j, int r, int c) -> double {
        int dr = (r - t.u0[j]) & (n0 - 1), dc = (c - t.u1[j]) & (n1 - 1);
        if (dr >= kWin || dc >= kWin) return 0.0;
        return (double)(W)t.psi[(size_t)j * 2 * kWin + dr] *
               (double)(W)t.psi[(size_t)j * 2 * kWin + kWin + dc];
    };
    // ---- trafo entries
    const size_t nE = L.ent.size();
    std::vector<std::map<long, double>> tr(M);
    std::vector<std::vector<int>> slots(M);
    for (int b = 0; b < L.nblk; b++)
        for (int e = L.blk_off[b]; e < L.blk_off[b + 1]; e++) {
            int j = L.ent[e] / 8, slot = L.ent[e] % 8;
            slots[j].push_back(slot);
            int rb = L.ent_rb[e], cl0 = L.ent_cc[e] & 255, cnt = (L.ent_cc[e] >> 8) & 255;
            // the parity bit names the window's first row: its weight at rb
            // is zero when the window starts at rb + 1
            int odd = L.ent_cc[e] >> 16;
            if (odd != (t.u0[j] & 1)) return 34;
            for (int q = 0; q < cnt; q++) {
                int c = b * L.BC + ((cl0 + q) & (L.BC - 1));
                double wc = (double)L.ent_q1.data()[(size_t)q * nE + e];
                for (int i = 0; i < 16; i++) {
                    double wr = (double)L.ent_qa.data()[(size_t)i * nE + e];
                    if (wr == 0.0 || wc == 0.0) continue;
                    int r = (rb + i) & (n0 - 1);
                    tr[j][(long)r * n1 + c] += wr * wc;
                }
            }
        }
    // the first row and the 16 row weights depend on the node only
    {
        std::vector<int> first(M, -1);
        for (size_t e = 0; e < nE; e++) {
            int j = L.ent[e] / 8;
            if (first[j] < 0) { first[j] = (int)e; continue; }
            size_t f = (size_t)first[j];
            if (L.ent_rb[e] != L.ent_rb[f]) return 32;
            for (int i = 0; i < 16; i++)
                if (L.ent_qa.data()[(size_t)i * nE + e] != L.ent_qa.data()[(size_t)i * nE + f])
                    return 33;
        }
    }
    for (int j = 0; j < M; j++) {
        if ((int)slots[j].size() != L.nslots[j] || L.nslots[j] > L.smax) return 30;
        std::vector<int> seen(8, 0);
        for (int s : slots[j]) if (s >= L.nslots[j] || seen[s]++) return 31;
    }
    // ---- adjoint tile entries
    const int R = L.R, Wn = R + L.BCa, nb = L.nbands;
    std::vector<std::map<long, double>> ad(M);
    {
        const size_t ntiles = (size_t)L.nblka * nb;
        if (L.band_ord.size() != ntiles) return 42;
        std::vector<int> once(ntiles, 0);
        int prev_len = 1 << 30;
        for (size_t k = 0; k < ntiles; k++) {
            int tile = L.band_ord[k];
            if (tile < 0 || (size_t)tile >= ntiles || once[tile]++) return 43;  // each tile once
            int b = tile / nb, v = tile - b * nb, lo = L.band_off[tile], hi = L.band_off[tile + 1];
            if (hi - lo > prev_len) return 40;     // longest first
            prev_len = hi - lo;
            for (int e = lo; e < hi; e++) {
                if (e > lo && L.band_node[e] <= L.band_node[e - 1]) return 41;  // ascending
                int j = L.band_node[e];
                const W *w = L.band_w.data() + (size_t)e * Wn;
                for (int rr = 0; rr < R; rr++)
                    for (int cc = 0; cc < L.BCa; cc++) {
                        double p = (double)w[rr] * (double)w[R + cc];
                        if (p == 0.0) continue;
                        ad[j][(long)(v * R + rr) * n1 + b * L.BCa + cc] += p;
                    }
            }
        }
    }
    // ---- both against the window, point by point
    for (int j = 0; j < M; j++) {
        int npts = 0;
        for (int s = 0; s < kWin; s++)
            for (int u = 0; u < kWin; u++) {
                int r = (t.u0[j] + s) & (n0 - 1), c = (t.u1[j] + u) & (n1 - 1);
                double want = expect(j, r, c);
                if (want == 0.0) continue;
                npts++;
                long key = (long)r * n1 + c;
                auto a = tr[j].find(key), d = ad[j].find(key);
                if (a == tr[j].end() || a->second != want) return 50;
                if (d == ad[j].end() || d->second != want) return 51;
            }
        if ((int)tr[j].size() != npts) return 52;  // no point outside the window
        if ((int)ad[j].size() != npts) return 53;
    }
    return 0;
}

// grid path: per ty x tx tile, the nodes whose window meets it, ascending
static int check_tiles(int N, int M, unsigned seed)
{
    std::mt19937 g(seed);
    std::uniform_real_distribution<double> U(-0.5, 0.5);
    std::vector<double> x(2 * (size_t)M);
    for (auto &v : x) v = U(g);
    x[0] = -0.5; x[1] = 0.5 - 1e-9;
    NfftTables t;
    if (build_nfft_tables(N, N, M, x.data(), 16, 16, &t)) return 60;
    std::vector<int> off, nodes;
    build_tile_lists(t, &off, &nodes);
    const int n0 = t.n0, n1 = t.n1, ty = t.ty, tx = t.tx;
    const int nty = (n0 + ty - 1) / ty, ntx = (n1 + tx - 1) / tx;
    if ((int)off.size() != nty * ntx + 1) return 61;
    for (int a = 0; a < nty; a++)
        for (int b = 0; b < ntx; b++) {
            int tile = a * ntx + b;
            std::vector<int> want;
            for (int j = 0; j < M; j++) {
                bool hit = false;
                for (int s = 0; s < kWin && !hit; s++)
                    for (int u = 0; u < kWin && !hit; u++) {
                        int r = (t.u0[j] + s) & (n0 - 1), c = (t.u1[j] + u) & (n1 - 1);
                        hit = r / ty == a && c / tx == b;
                    }
                if (hit) want.push_back(j);
            }
            std::vector<int> got(nodes.begin() + off[tile], nodes.begin() + off[tile + 1]);
            if (got != want) return 62;
        }
    return 0;
}

int main()
{
    if (int r = check_tiles(24, 200, 7)) { std::printf("tiles %d\n", r); return 1; }
    if (int r = check_tiles(56, 300, 8)) { std::printf("tiles %d\n", r); return 1; }
    struct Case { int N, M, BC; bool pair; unsigned seed; };
    const Case cases[] = {{24, 300, 4, true, 1}, {24, 300, 2, true, 2}, {40, 500, 4, false, 3},
                          {8, 60, 16, true, 4}, {96, 400, 4, true, 5}};
    int k = 0;
    for (const Case &c : cases) {
        int rf = check<float>(c.N, c.M, c.BC, c.pair, c.seed);
        int rd = check<double>(c.N, c.M, c.BC, c.pair, c.seed + 100);
        if (rf || rd) {
            std::printf("case %d: float %d double %d\n", k, rf, rd);
            return 1;
        }
        k++;
    }
    std::printf("ok\n");
    return 0;
}
"""


def test_fused_lists_reproduce_every_window(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    src = tmp_path / "h.cpp"
    src.write_text(HARNESS)
    exe = tmp_path / "h"
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", CSRC, str(src),
                    os.path.join(CSRC, "tables.cpp"), "-o", str(exe), "-pthread"], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "ok" in r.stdout, (r.returncode, r.stdout, r.stderr)
