// tables.h -- host FP64 tables of the NUDIM engine (node geometry, Kaiser-
// Bessel window, deconvolution factors, spreading tile lists, CGNR weights,
// polar-line classification, the GSL-default random fill).
#pragma once

#include <cstddef>
#include <cstdint>
#include <memory>
#include <vector>

namespace nudim {

constexpr double kRefPi = 3.1415926;               // src/grid.h:11
constexpr double kTruePi = 3.14159265358979323846; // NFFT window constants

int grid_size(int N);  // n = 2 * next_pow2(N) (reconstruction.c:316, 390)

// src/grid.c:84 / 78-97 / 100-133
int equal_angle_count(double amin, double amax, double ainterval);
void equal_angle_sample_2d(double amin, double amax, double ainterval, int nx, double *x);
// The same node set in factored form: radii r[nx] (angle-independent) and the
// lines' sin / cos (sg, cg: equal_angle_count(amin, amax, ainterval) each).
void polar_factors(double amin, double amax, double ainterval, int nx, double *r, double *sg,
                   double *cg);
void uniform_sample_2d(int nx, int nz, double *x);
// src/reconstruction.c:375-384
int polar_lines(double gam_min, double interval, double padangle, double *pad_min,
                double *pad_max);

struct NfftTables {
    int N0 = 0, N1 = 0, n0 = 0, n1 = 0, M = 0;
    std::vector<int> u0, u1;          // first window index per node (may be < 0)
    std::vector<double> psi;          // M x (2*kW): psi0[0..kW), psi1[0..kW)
    std::vector<double> c0, c1;       // 1 / (n * phi_hat(k)), centred k
    // tiles of the grid path's spreading gather (lists: build_tile_lists)
    int ty = 16, tx = 16, nty = 0, ntx = 0;
};

int build_nfft_tables(int N0, int N1, int M, const double *x, int ty, int tx, NfftTables *t);

// Work lists of the fused NFFT (column blocks of BC columns of the n0 x n1
// oversampled grid):
//   trafo:   per block, the nodes whose window columns meet the block, each
//            with its partial slot (0 = the node's first block, 1, ...);
//   adjoint: column blocks of BCa columns; per tile of R = 32 / BCa rows x
//            BCa columns (one grid point per warp lane), the nodes whose
//            window meets the tile, ascending.
template <typename W> struct HostArray {  // uninitialised until written
    std::unique_ptr<W[]> p;
    size_t n = 0;
    void alloc(size_t k) { p.reset(new W[k ? k : 1]); n = k; }
    W *data() { return p.get(); }
    const W *data() const { return p.get(); }
    size_t size() const { return n; }
};

// W: the element type of the weights (the plan's precision).
template <typename W> struct FusedLists {
    int BC = 0, nblk = 0, smax = 0;
    int BCa = 0, nblka = 0, R = 0, nbands = 0;
    std::vector<int> blk_off, ent;          // ent = node * 8 + slot
    std::vector<unsigned char> nslots;      // blocks per node
    // per trafo entry (structure of arrays over the entries): even first
    // window row, cl0 | cnt << 8 | odd << 16 (odd: the window's first row is
    // rb + 1), 16 aligned row weights, nq column weights
    int nq = 0;
    std::vector<int> ent_rb, ent_cc;
    HostArray<W> ent_qa, ent_q1;
    std::vector<int> band_off, band_node;   // CSR over tiles b * nbands + v
    HostArray<W> band_w;                    // per entry R row + BCa column weights
    std::vector<int> band_ord;              // every tile once, longest list first
};

// BC a power of two dividing n1; BCa a power of two <= 32 dividing n1.
// Returns 0, -1 (bad shape) or -2 (a window meets one trafo block twice:
// the grid is too narrow for column blocks of BC).  adjoint = false leaves
// the adjoint lists without entries (band_off = band_node = {0}, no
// weights): a plan that only runs the trafo.
template <typename W>
int build_fused_lists(const NfftTables &t, int BC, int BCa, bool pair_rows, FusedLists<W> *L,
                      bool adjoint = true);

// Spreading tile lists of the grid path: node ids whose window touches each
// ty x tx tile of the n0 x n1 grid, ascending, CSR layout.
void build_tile_lists(const NfftTables &t, std::vector<int> *off, std::vector<int> *nodes);

// e^{-2 pi i k / n}, k < n, interleaved (re, im)
void fft_twiddles(int n, std::vector<double> *tw);

// reconstruction.c:415-426 (--weight)
void cgnr_weights(int A, int np, double padangle, double *w);

// reconstruction.c:437-484: per polar line a, known[a] = 1 when the line is
// a measured tilt outside the cross-validation band, order[a] = tilt index.
void classify_lines(double pad_min, double padangle, double gam_min, double gam_max,
                    double interval, int A, std::vector<int> *known, std::vector<int> *order);

// gsl_rng_uniform with gsl_rng_default (MT19937, seed 0 -> 4357).
void mt19937_uniform(uint32_t seed, size_t n, double *out);

}  // namespace nudim
