"""CPU restatement of PCAone's randomized-SVD path (the oracle).

TEST INFRASTRUCTURE ONLY.  Nothing in the product imports this module; only
tests, the smoke check and the CPU-baseline leg of the benchmark use it, and
only as a checker / baseline.  It is pinned against the reference itself (the
reference's own sources compiled by oracle/Makefile and run by
oracle/ref_driver.cpp) through the fixtures under tests/golden/.

The restatement follows the reference in its own orientation: the data
matrix ``X`` is N x M (samples x SNPs, ``Data::G`` in src/Data.hpp:50) in
float64, and every step below cites the reference file:line it restates.
Dense linear algebra uses numpy/LAPACK: ``numpy.linalg.qr`` is a Householder
QR with the same reflector sign rule as Eigen's HouseholderQR (beta =
-sign(alpha) * norm), so the Q factors agree column by column.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from typing import Optional

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIBDIR = os.path.join(_HERE, "lib")
_RNG_SO = os.path.join(_LIBDIR, "liboracle_rng.so")

# src/Common.hpp:58-59 and src/Data.hpp:7
BED_MISSING_VALUE = -9.0
BED2GENO = np.array([1.0, BED_MISSING_VALUE, 0.5, 0.0])
VAR_TOL = 1e-9


# ----------------------------------------------------------------------------
# libstdc++ random streams (src/Halko.cpp:15-23, src/RSVD.hpp:54-78)
# ----------------------------------------------------------------------------
def _native_flag() -> str:
    """The reference builds with -march=native (-mcpu=native on Arm), which lets
    the compiler contract the polar method's arithmetic into FMAs; the same flag
    here keeps the random stream identical to the reference built on this host."""
    import platform
    return "-mcpu=native" if platform.machine() in ("aarch64", "arm64") else "-march=native"


def build_rng_lib(force: bool = False) -> str:
    """Compile oracle/stdrng.cpp into oracle/lib/liboracle_rng.so."""
    src = os.path.join(_HERE, "stdrng.cpp")
    if force or not os.path.exists(_RNG_SO) or os.path.getmtime(_RNG_SO) < os.path.getmtime(src):
        os.makedirs(_LIBDIR, exist_ok=True)
        tmp = _RNG_SO + f".tmp{os.getpid()}"
        subprocess.check_call(["g++", "-O3", "-std=c++17", _native_flag(), "-shared", "-fPIC", src, "-o", tmp])
        os.replace(tmp, _RNG_SO)
    return _RNG_SO


_rng_lib = None


def _lib():
    global _rng_lib
    if _rng_lib is None:
        _rng_lib = ctypes.CDLL(build_rng_lib())
        _rng_lib.oracle_random_omega.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int64,
                                                  ctypes.c_int64, ctypes.c_void_p]
        _rng_lib.oracle_shuffle_columns.argtypes = [ctypes.c_int64, ctypes.c_void_p]
    return _rng_lib


def random_omega(seed: int, rows: int, cols: int, gaussian: bool = True) -> np.ndarray:
    """Omega (rows x cols) exactly as RsvdOpData::initOmg draws it (src/Halko.cpp:15-23)."""
    out = np.empty((rows, cols), dtype=np.float64, order="F")
    _lib().oracle_random_omega(int(seed), 1 if gaussian else 0, rows, cols, out.ctypes.data)
    return out


def shuffle_columns(n: int) -> np.ndarray:
    """The in-core column order of PCAone::permute_matrix (src/RSVD.hpp:61-70)."""
    out = np.empty(n, dtype=np.int32)
    _lib().oracle_shuffle_columns(n, out.ctypes.data)
    return out


def genovec_to_bed(genovec: np.ndarray, nsamples: int) -> np.ndarray:
    """PLINK 2 hard calls (2-bit ALT allele counts, 3 = missing: what pgenlib's
    ReadHardcalls reports as 0, 1, 2, -3) as PLINK 1 codes with A1 = ALT, so
    that BED2GENO gives the dosage FilePgen uses, v / 2 (src/FilePgen.cpp:16-21):
    2 -> 00 (1.0), 1 -> 10 (0.5), 0 -> 11 (0.0), 3 -> 01 (missing)."""
    g = np.asarray(genovec, dtype=np.uint8)
    lut = np.array([3, 2, 0, 1], dtype=np.uint8)
    out = np.zeros_like(g)
    for s in range(4):
        out |= lut[(g >> (2 * s)) & 3] << (2 * s)
    return out


def permute_plink_order(nsnps: int, nsamples: int, bands: int, buffer_gb: int = 2) -> np.ndarray:
    """The SNP order of the reference's out-of-core window method: order[p] is
    the .bed row that permute_plink (src/FilePlink.cpp:303-408) writes at row
    p of the rewritten file.  Restated from its index arithmetic (ia -> ib,
    :383-393), without the file I/O: buffers of twoGB_snps SNPs (:311-314),
    band starts bandidx (:328-341), a shorter last buffer (:365-374)."""
    bps = (nsamples + 3) // 4
    two_gb_snps = min(int(np.floor(1073741824.0 * buffer_gb / bps)), nsnps)
    bufsize = two_gb_snps // bands
    two_gb_snps = bufsize * bands
    bufidx = bufsize
    nblocks = (nsnps + two_gb_snps - 1) // two_gb_snps
    modr2 = nsnps % two_gb_snps
    modr, bandsize = nsnps % bands, (nsnps + bands - 1) // bands
    bandidx = [i * bandsize if (modr == 0 or i < modr) else modr * bandsize + (bandsize - 1) * (i - modr)
               for i in range(bands)]
    order = np.full(nsnps, -1, dtype=np.int64)
    for i in range(nblocks):
        if i == nblocks - 1 and modr2 != 0:
            snps2 = nsnps - (nblocks - 1) * two_gb_snps
            bufsize = (snps2 + bands - 1) // bands
            modr2 = snps2 % bands
        for b in range(bands):
            last = bufsize - 1
            take_last = i != nblocks - 1 or b < modr2 or modr2 == 0
            for j in range(last + (1 if take_last else 0)):
                order[i * bufidx + bandidx[b] + j] = i * two_gb_snps + j * bands + b
    assert (order >= 0).all() and len(set(order.tolist())) == nsnps
    return order


# ----------------------------------------------------------------------------
# PLINK decode, counts, allele frequency (src/FilePlink.cpp:26-110)
# ----------------------------------------------------------------------------
def unpack_codes(packed: np.ndarray, nsamples: int) -> np.ndarray:
    """(M, ceil(N/4)) bytes -> (M, N) 2-bit codes; padding lanes dropped
    (the ``j < nsamples`` guard of src/FilePlink.cpp:42,77)."""
    p = np.asarray(packed, dtype=np.uint8)
    codes = np.stack([(p >> s) & 3 for s in (0, 2, 4, 6)], axis=-1).reshape(p.shape[0], -1)
    return codes[:, :nsamples]


def bed_counts(packed: np.ndarray, nsamples: int) -> np.ndarray:
    """Per-SNP counts of the four codes, columns (n00, n01, n10, n11) = (two A1
    copies, missing, heterozygous, no A1 copy)."""
    codes = unpack_codes(packed, nsamples)
    return np.stack([(codes == c).sum(axis=1) for c in range(4)], axis=1).astype(np.int64)


def allele_freq(counts: np.ndarray) -> np.ndarray:
    """F_j = sum of BED2GENO over observed genotypes / n_observed, 0 if none
    (src/FilePlink.cpp:37-55).  The sum of 1.0 and 0.5 terms is exact in double,
    so n00 + 0.5*n10 reproduces the reference's running sum bit for bit."""
    n00, n10, n11 = counts[:, 0], counts[:, 2], counts[:, 3]
    c = n00 + n10 + n11
    s = n00.astype(np.float64) + 0.5 * n10.astype(np.float64)
    with np.errstate(invalid="ignore", divide="ignore"):
        f = s / c.astype(np.float64)
    return np.where(c == 0, 0.0, f)


def maf_keep(F: np.ndarray, maf: float) -> np.ndarray:
    """Data::filter_snps_resize_F (src/Data.cpp:88-105): the SNPs whose minor
    allele frequency (MAF macro, src/Common.hpp:26) exceeds maf, in file order."""
    F = np.asarray(F, dtype=np.float64)
    return np.flatnonzero(np.where(F > 0.5, 1.0 - F, F) > maf).astype(np.int64)


def decode_centered(packed: np.ndarray, nsamples: int, F: np.ndarray):
    """X (N x M) = BED2GENO[code] - F_j with missing entries set to 0 (mean
    imputation), and the missing mask C (M x N, bool); src/FilePlink.cpp:71-110."""
    codes = unpack_codes(packed, nsamples)             # (M, N)
    miss = codes == 1
    g = BED2GENO[codes] - F[:, None]
    g[miss] = 0.0
    return np.asfortranarray(g.T), miss


def standardize_scale(F: np.ndarray, ploidy: int = 2) -> np.ndarray:
    """Per-SNP factor sqrt(ploidy)/sqrt(f(1-f)) when sd > VAR_TOL, else 1
    (src/Data.cpp:351-362)."""
    sd = np.sqrt(F * (1.0 - F))
    with np.errstate(divide="ignore"):
        s = np.sqrt(float(ploidy)) / sd
    return np.where(sd > VAR_TOL, s, 1.0)


# ----------------------------------------------------------------------------
# small utilities (src/RSVD.hpp:80-89, src/Utils.cpp:118-200)
# ----------------------------------------------------------------------------
def flip_omg(omg2: np.ndarray, omg: np.ndarray) -> None:
    """PCAone::flipOmg: flip column i of omg if ||omg2_i - omg_i||_1 >
    2 ||omg2_i + omg_i||_1, then omg2 <- omg (in place)."""
    a = np.abs(omg2 - omg).sum(axis=0)
    b = np.abs(omg2 + omg).sum(axis=0)
    omg[:, a > 2 * b] *= -1.0
    omg2[...] = omg


def mev(X: np.ndarray, Y: np.ndarray) -> float:
    """Mean explained variance, src/Utils.cpp:194-200."""
    return float(np.linalg.norm(X.T @ Y, axis=0).sum() / X.shape[1])


def flip_uv(U: np.ndarray, V: np.ndarray, ubase: bool = False) -> None:
    """flip_UV (src/Utils.cpp:118-154) for V with the same column count as U."""
    base = U if ubase else V
    idx = np.abs(base).argmax(axis=0)
    neg = base[idx, np.arange(base.shape[1])] < 0
    U[:, neg] *= -1.0
    V[:, neg] *= -1.0


def householder_q(A: np.ndarray) -> np.ndarray:
    """Thin Q of a Householder QR (Eigen HouseholderQR::householderQ()*I)."""
    return np.linalg.qr(A, mode="reduced")[0]


# ----------------------------------------------------------------------------
# the data object (src/Data.hpp:9-59) restricted to the in-core PLINK path
# ----------------------------------------------------------------------------
class OracleData:
    def __init__(self, packed: np.ndarray, nsamples: int, *, emu: bool = False, perm: bool = False,
                 seed: int = 112, bands: int = 64, rand: int = 1, ploidy: int = 2,
                 svd_t: int = 2, mev_metric: bool = True, omega0: Optional[np.ndarray] = None):
        self.nsamples = int(nsamples)
        self.nsnps = int(packed.shape[0])
        self.counts = bed_counts(packed, nsamples)
        self.F = allele_freq(self.counts)
        self.G, self.C = decode_centered(packed, nsamples, self.F)
        self.emu = emu
        self.missme = emu
        self.perm = perm
        self.perm_idx: Optional[np.ndarray] = None
        self.seed = seed
        self.bands = bands
        self.rand = rand
        self.ploidy = ploidy
        self.svd_t = svd_t      # 1: single-pass sSVD, 2: window-based winSVD
        self.mev = mev_metric
        # an explicit initial test matrix replaces the libstdc++ draw (used to
        # feed the reference's own Omega into the restatement)
        self.omega0 = None if omega0 is None else np.asfortranarray(omega0, dtype=np.float64)

    @classmethod
    def from_dense(cls, values: np.ndarray, *, perm: bool = False, seed: int = 112, bands: int = 64,
                   rand: int = 1, svd_t: int = 2, omega0: Optional[np.ndarray] = None) -> "OracleData":
        """FileBinary input (src/FileBinary.cpp:54-64): values M x N (float32
        as read), each SNP centred by its mean in float64; run with -C 0, so
        standardize_E does nothing (src/Data.cpp:353)."""
        self = cls.__new__(cls)
        v = np.asarray(values, dtype=np.float32)
        self.nsnps, self.nsamples = int(v.shape[0]), int(v.shape[1])
        self.counts = None
        self.F = None
        G = v.T.astype(np.float64)
        self.G = np.asfortranarray(G - G.mean(axis=0)[None, :])
        self.C = np.zeros((self.nsnps, self.nsamples), dtype=bool)
        self.emu = self.missme = False
        self.perm = perm
        self.perm_idx = None
        self.seed, self.bands, self.rand, self.ploidy = seed, bands, rand, 2
        self.svd_t = svd_t
        self.mev = True
        self.omega0 = None if omega0 is None else np.asfortranarray(omega0, dtype=np.float64)
        return self

    def standardize_E(self) -> None:
        """src/Data.cpp:351-362: column i scaled with F(i) (column order as is);
        nothing for FileBinary input run with -C 0."""
        if self.F is None:
            return
        self.G *= standardize_scale(self.F, self.ploidy)[None, :]

    def fit_with_pi(self, U: np.ndarray, S: np.ndarray, VT: np.ndarray) -> None:
        """EMU fill of missing entries, src/Data.cpp:318-348.

        Missing entry (sample j, column i) <- clamp(sum_k U_jk S_k VT_ki, -F(i), 1-F(i)).
        With permuted columns the mask is looked up at the original column
        perm[i] but the clamp uses F(i) of the unpermuted order, as the
        reference does (src/Data.cpp:322,328)."""
        fit = (U * S[None, :]) @ VT                      # N x M
        if self.perm and self.perm_idx is not None:
            mask = self.C[self.perm_idx, :].T           # N x M in the permuted order
        else:
            mask = self.C.T
        lo = -self.F[None, :]
        hi = 1.0 - self.F[None, :]
        filled = np.minimum(np.maximum(fit, lo), hi)
        self.G[mask] = filled[mask]


# ----------------------------------------------------------------------------
# RSVD operators (src/Halko.hpp, src/Halko.cpp)
# ----------------------------------------------------------------------------
class RsvdOp:
    def __init__(self, data: OracleData, k: int, os_: int):
        self.data = data
        self.nk = int(k)
        self.os = int(os_)
        self.size = self.nk + self.os
        self.update = False
        self.standardize = False
        self.U = self.V = self.S = None
        self.epochs_run = 0
        self.init_omg()

    def rows(self):
        return self.data.nsnps

    def cols(self):
        return self.data.nsamples

    def init_omg(self):
        """src/Halko.cpp:15-23."""
        if self.data.omega0 is not None:
            self.Omg = self.data.omega0.copy(order="F")
        else:
            self.Omg = random_omega(self.data.seed, self.cols(), self.size, gaussian=bool(self.data.rand))
        self.Omg2 = self.Omg.copy()

    def set_flags(self, update: bool, standardize: bool):
        self.update, self.standardize = update, standardize

    def compute_g_and_h(self, pi: int):
        raise NotImplementedError

    def compute_usv(self, p: int, tol: float):
        """RsvdOpData::computeUSV, src/Halko.cpp:46-97."""
        nk = self.nk
        Upre = None
        Ucur = None
        pi = 0
        self.epochs_run = 0
        while pi <= p:
            G, H = self.compute_g_and_h(pi)
            self.epochs_run += 1
            Q1, R1 = np.linalg.qr(G, mode="reduced")
            Q2, R2 = np.linalg.qr(Q1, mode="reduced")
            R = R2 @ R1
            B = np.linalg.solve(R.T, H.T)                   # R^T B = H^T
            UB, s, VBt = np.linalg.svd(B, full_matrices=False)
            Ucur = VBt.T[:, :nk]
            if pi > 0:
                if self.data.mev:
                    diff = 1.0 - mev(Ucur, Upre)
                else:
                    raise NotImplementedError("minSSE convergence")
                if diff < tol or pi == p:
                    if self.data.svd_t == 2 and 2 ** pi < self.data.bands:
                        p = int(np.log2(self.data.bands))
                    else:
                        self.U = Ucur
                        self.V = Q2 @ UB[:, :nk]
                        self.S = s[:nk].copy()
                        break
                else:
                    Upre = Ucur
            else:
                Upre = Ucur
            pi += 1
        self.U = Ucur
        return self


class NormalRsvdOp(RsvdOp):
    """NormalRsvdOpData::computeGandH in-core branch, src/Halko.cpp:99-128."""

    def compute_g_and_h(self, pi: int):
        d = self.data
        if pi == 0:
            self.init_omg()
            if self.update:
                d.fit_with_pi(self.U, self.S, self.V.T)
            if self.standardize:
                d.standardize_E()
        if pi > 0:
            self.Omg = householder_q(self.H)
            flip_omg(self.Omg2, self.Omg)
        G = d.G.T @ self.Omg
        self.H = d.G @ G
        return G, self.H


class FancyRsvdOp(RsvdOp):
    """FancyRsvdOpData::computeGandH in-core branch, src/Halko.cpp:155-225."""

    def __init__(self, data: OracleData, k: int, os_: int):
        super().__init__(data, k, os_)
        self.H1 = np.zeros((self.cols(), self.size))
        self.H2 = np.zeros((self.cols(), self.size))
        self.bandsize = 1
        self.blocksize = 0
        self.H = np.zeros((self.cols(), self.size))

    def compute_g_and_h(self, pi: int):
        d = self.data
        bands = d.bands
        if pi == 0:
            self.init_omg()
        if 2 ** pi >= bands:
            self.H1[...] = 0.0
            self.H2[...] = 0.0
        if pi == 0:
            if self.update:
                d.fit_with_pi(self.U, self.S, self.V.T)
            if self.standardize:
                d.standardize_E()
            self.bandsize = 1
            self.blocksize = int(np.ceil(d.nsnps / bands))
            if d.perm and not (self.update and d.emu):
                d.perm_idx = shuffle_columns(d.nsnps)
                d.G = np.asfortranarray(d.G[:, d.perm_idx])
        self.bandsize = min(self.bandsize * 2, bands)
        G = np.empty((d.nsnps, self.size))
        bs = self.blocksize
        i = 1
        for b in range(bands):
            start = b * bs
            stop = d.nsnps - 1 if (b + 1) * bs >= d.nsnps else (b + 1) * bs - 1
            Xb = d.G[:, start:stop + 1]
            G[start:stop + 1] = Xb.T @ self.Omg
            if i <= self.bandsize // 2:
                self.H1 += Xb @ G[start:stop + 1]
            else:
                self.H2 += Xb @ G[start:stop + 1]
            adjacent = pi > 0 and (b + 1) == 2 ** (pi - 1) and 2 ** pi < bands
            if (b + 1) < self.bandsize and not adjacent:
                i += 1
                continue
            if not (i == self.bandsize or i == self.bandsize // 2 or adjacent):
                i += 1
                continue
            self.H = self.H1 + self.H2
            self.Omg = householder_q(self.H)
            flip_omg(self.Omg2, self.Omg)
            if i == self.bandsize:
                self.H1[...] = 0.0
                i = 0
            else:
                self.H2[...] = 0.0
            i += 1
        return G, self.H


def run_pca_with_halko(data: OracleData, k: int, oversamples: int, maxp: int = 20, tol: float = 1e-4,
                       maxiter: int = 100, tolem: float = 1e-5):
    """run_pca_with_halko, src/Halko.cpp:271-320 (PLINK, non-LD, non-PCAngsd).

    ``oversamples`` is used as given (the CLI raises it to at least k,
    src/Cmd.cpp:216; callers that mirror the CLI pass max(p, k))."""
    op = (FancyRsvdOp if data.svd_t == 2 else NormalRsvdOp)(data, k, oversamples)
    em_iters = 0
    if not data.missme:
        op.set_flags(False, True)
        op.compute_usv(maxp, tol)
    else:
        op.set_flags(False, False)
        op.compute_usv(maxp, tol)
        flip_uv(op.U, op.V)
        for it in range(maxiter):
            op.set_flags(True, False)
            Vpre = op.V.copy()
            op.compute_usv(maxp, tol)
            flip_uv(op.U, op.V)
            diff = 1.0 - mev(op.V, Vpre)
            em_iters = it + 1
            if diff < tolem:
                break
        if data.emu:
            op.set_flags(True, True)
            op.compute_usv(maxp, tol)
            flip_uv(op.U, op.V)
    op.em_iters = em_iters
    return op


def project(packed_new: np.ndarray, nsamples: int, F: np.ndarray, V: np.ndarray, S: np.ndarray, mode: int,
            ploidy: int = 2) -> np.ndarray:
    """Scores of new samples on a fit (run_projection, src/Projection.cpp:236-247).

    The new genotypes are decoded and centred with the fit's allele
    frequencies F (read from the .mbim, src/Data.cpp:17-32) and standardised
    with them; V (M x k, file order) and S are the fit's loadings and
    singular values.  mode 1: U = G V S^-1 (missing genotypes at the mean);
    mode 2: per sample the least-squares solution of (V S) x = g over its
    observed SNPs (solve_projection_scores, src/Projection.cpp:159-178)."""
    G, C = decode_centered(packed_new, nsamples, F)
    G = G * standardize_scale(F, ploidy)[None, :]
    if mode == 1:
        return G @ (V / S[None, :])
    VS = V * S[None, :]
    U = np.zeros((nsamples, V.shape[1]))
    for i in range(nsamples):
        obs = ~C[:, i]
        U[i] = np.linalg.lstsq(VS[obs], G[i, obs], rcond=None)[0]
    return U


def arnoldi_matvec(data: OracleData, x: np.ndarray) -> np.ndarray:
    """y = X (X^T x) summed over SNP blocks (ArnoldiOpData::perform_op,
    src/Arnoldi.cpp:18-46)."""
    return data.G @ (data.G.T @ x)


# ----------------------------------------------------------------------------
# comparison metrics
# ----------------------------------------------------------------------------
def sin_largest_angle(A: np.ndarray, B: np.ndarray) -> float:
    """sin of the largest principal angle between span(A) and span(B),
    computed as ||(I - QaQa^T) Qb||_2 (no arccos of cosines near 1)."""
    Qa = np.linalg.qr(A)[0]
    Qb = np.linalg.qr(B)[0]
    R = Qb - Qa @ (Qa.T @ Qb)
    return float(np.linalg.norm(R, 2))


def eig_relerr(Sa: np.ndarray, Sb: np.ndarray) -> np.ndarray:
    return np.abs(Sa ** 2 - Sb ** 2) / np.abs(Sb ** 2)


def well_separated(S: np.ndarray, gap: float = 0.05) -> int:
    """Number of leading components whose squared singular value is separated
    from the next by a relative gap above ``gap``; principal angles are compared
    on these (near-degenerate noise components are not determined by 7 power
    iterations, neither in the reference nor here)."""
    e = S ** 2
    n = 0
    for i in range(len(e) - 1):
        if (e[i] - e[i + 1]) / e[i] > gap:
            n = i + 1
    return n
