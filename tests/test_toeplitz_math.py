"""The arithmetic behind the mixed form's CGNR by Toeplitz embedding
(nudim_gb300/csrc/nfft_fused.cu: k_toep_gtable, k_toep_circ, k_col_toeplitz;
ops.cu: cgnr_run_toeplitz), restated in numpy on small cases:

  - T = A^H W A applied as crop(IDFT(DFT(circulant of K) * DFT(pad(p)))) on an
    nt x nt circulant with nt >= 2N - 1 equals the direct NDFT product
    (A the trafo f_j = sum_k fhat_k e^{-2 pi i k.x_j}, src/reconstruction.c:571);
  - the kernel K[m] = sum_j w_j e^{2 pi i m.x_j} from the polar set's factors
    (radial sum G tabulated at spacing 1/32, 8-point Lagrange interpolation,
    the kernel's node offsets and denominators) is within 1e-11 of the direct
    sum;
  - the inverse four-step split used after the product (thread k1 holds
    Y[k1 + R1 k2]; R2-point DFTs over k2, twiddle e^{+2 pi i k1 t2 / n},
    R1-point DFTs over k1, output t2 + R2 t1) is the inverse DFT, for the
    24 x 32 and 32 x 32 splits;
  - CG on the normal equations with z' = z - alpha T p gives the iterates of
    the node-space recursion (r -= alpha A p, z' = A^H W r)."""
import numpy as np

PI = 3.1415926  # the reference's grid.h


def polar(npx, A, padangle, amin):
    ang = amin - padangle
    sg, cg = [], []
    for _ in range(A):
        ang += padangle
        sg.append(np.sin(ang / 180 * PI))
        cg.append(np.cos(ang / 180 * PI))
    step, rr, r = 1.0 / npx, -0.5 - 1.0 / npx, []
    for _ in range(npx):
        rr += step
        r.append(rr)
    h = npx // 2
    w = np.where(np.arange(npx) == h, PI / (4 * A * h * h),
                 padangle / 180 * PI * np.abs(np.arange(npx) - h) / (h * h))
    return np.array(r), np.array(sg), np.array(cg), w


def ndft_ops(N, x0, x1, w):
    k = np.arange(N) - N // 2
    K0, K1 = np.meshgrid(k, k, indexing="ij")
    E = np.exp(-2j * np.pi * (np.outer(x0, K0.ravel()) + np.outer(x1, K1.ravel())))
    A = lambda f: E @ f.ravel()
    AH = lambda r: (E.conj().T @ r).reshape(N, N)
    return A, lambda p: AH(w * A(p))


def kernel_direct(N, x0, x1, w):
    m = np.arange(-N + 1, N)
    return np.array([(np.exp(2j * np.pi * (m0 * x0[None, :] + m[:, None] * x1[None, :])) * w)
                     .sum(1) for m0 in m])  # [m0 + N - 1][m1 + N - 1]


def kernel_interp(N, r, sg, cg, w):
    delta = 1 / 32
    K0 = int(np.ceil(2 * N / delta)) + 8
    sk = (np.arange(2 * K0 + 1) - K0) * delta
    G = (np.exp(2j * np.pi * np.outer(sk, r)) * w).sum(1)
    rden = np.array([-1 / 5040, 1 / 720, -1 / 240, 1 / 144, -1 / 144, 1 / 240, -1 / 720, 1 / 5040])
    m = np.arange(-N + 1, N)
    M0, M1 = np.meshgrid(m, m, indexing="ij")
    u = (M0[..., None] * sg + M1[..., None] * cg) / delta + K0
    fu = np.floor(u)
    t, k0 = u - fu, fu.astype(int) - 3
    d = [t - (j - 3) for j in range(8)]
    pre = [np.ones_like(t)]
    for j in range(1, 8):
        pre.append(pre[-1] * d[j - 1])
    suf = [None] * 7 + [np.ones_like(t)]
    for j in range(6, -1, -1):
        suf[j] = suf[j + 1] * d[j + 1]
    return sum((pre[j] * suf[j] * rden[j] * G[k0 + j]).sum(-1) for j in range(8))


def apply_circulant(K, N, nt, p):
    circ = np.zeros((nt, nt), complex)
    m = np.arange(-N + 1, N)
    circ[np.ix_(m % nt, m % nt)] = K
    khat = np.fft.fft2(circ) / nt ** 2
    k = np.arange(N) - N // 2
    P = np.zeros((nt, nt), complex)
    P[np.ix_(k % nt, k % nt)] = p
    Q = np.fft.ifft2(khat * np.fft.fft2(P)) * nt ** 2
    return Q[np.ix_(k % nt, k % nt)]


def test_circulant_product_is_the_normal_operator():
    N, A = 16, 37
    r, sg, cg, w1 = polar(N, A, 5.0, -90.0)
    x0, x1, w = np.outer(sg, r).ravel(), np.outer(cg, r).ravel(), np.tile(w1, A)
    _, T = ndft_ops(N, x0, x1, w)
    rng = np.random.default_rng(1)
    p = rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))
    K = kernel_direct(N, x0, x1, w)
    for nt in (2 * N, 2 * N + 16, 3 * N):  # any nt >= 2N - 1
        q = apply_circulant(K, N, nt, p)
        assert np.linalg.norm(q - T(p)) / np.linalg.norm(T(p)) < 1e-13


def test_interpolated_kernel_matches_the_direct_sum():
    N, A = 24, 61
    r, sg, cg, w1 = polar(N, A, 3.0, -90.0)
    x0, x1, w = np.outer(sg, r).ravel(), np.outer(cg, r).ravel(), np.tile(w1, A)
    Kd = kernel_direct(N, x0, x1, w)
    Ki = kernel_interp(N, r, sg, cg, w1)
    assert np.abs(Ki - Kd).max() / np.abs(Kd).max() < 1e-11


def test_inverse_four_step_split():
    rng = np.random.default_rng(2)
    for R1, R2 in ((24, 32), (32, 32), (16, 16)):
        n = R1 * R2
        Y = rng.standard_normal(n) + 1j * rng.standard_normal(n)
        Z = np.zeros((R1, R2), complex)
        for k1 in range(R1):
            Z[k1] = np.fft.ifft(Y[k1 + R1 * np.arange(R2)]) * R2
            Z[k1] *= np.exp(2j * np.pi * k1 * np.arange(R2) / n)
        y = np.zeros(n, complex)
        for t2 in range(R2):
            y[t2 + R2 * np.arange(R1)] = np.fft.ifft(Z[:, t2]) * R1
        assert np.abs(y - np.fft.ifft(Y) * n).max() < 1e-10 * np.abs(Y).sum() / n ** 0.5


def test_coefficient_space_cg_has_the_node_space_iterates():
    N, A = 12, 31
    r, sg, cg, w1 = polar(N, A, 6.0, -90.0)
    x0, x1, w = np.outer(sg, r).ravel(), np.outer(cg, r).ravel(), np.tile(w1, A)
    Aop, T = ndft_ops(N, x0, x1, w)
    AH = lambda v: (np.exp(2j * np.pi * (np.outer(
        (np.arange(N) - N // 2).repeat(N), x0) + np.outer(np.tile(np.arange(N) - N // 2, N), x1)))
        @ v).reshape(N, N)
    rng = np.random.default_rng(3)
    y = rng.standard_normal(len(x0)) + 1j * rng.standard_normal(len(x0))
    f0 = rng.standard_normal((N, N)).astype(complex)
    # node-space CGNR (the reference's solver)
    f, res = f0.copy(), y - Aop(f0)
    z = AH(w * res)
    p = z.copy()
    fr = []
    for _ in range(10):
        v = Aop(p)
        al = np.vdot(z, z).real / np.vdot(v, w * v).real
        f, res = f + al * p, res - al * v
        z2 = AH(w * res)
        p = z2 + np.vdot(z2, z2).real / np.vdot(z, z).real * p
        z = z2
        fr.append(f.copy())
    # coefficient space
    g, zc = f0.copy(), AH(w * y) - T(f0)
    pc = zc.copy()
    for k in range(10):
        q = T(pc)
        al = np.vdot(zc, zc).real / np.vdot(pc, q).real
        g, z2 = g + al * pc, zc - al * q
        pc = z2 + np.vdot(z2, z2).real / np.vdot(zc, zc).real * pc
        zc = z2
        assert np.linalg.norm(g - fr[k]) / np.linalg.norm(fr[k]) < 1e-9
