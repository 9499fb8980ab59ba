"""Host-side mirror of the reference's RSVD operator interface over the C-ABI.

Names and call order follow src/Halko.hpp / src/Halko.cpp so that code (and
tests) written against the reference read the same:

    data = FileBed("prefix")                 # FileBed ctor + Data::prepare (in-core)
    op = FancyRsvdOpData(data, k, os)        # or NormalRsvdOpData
    op.setFlags(False, True)
    op.computeUSV(maxp, tol)                 # -> op.U, op.S, op.V

Everything runs on the GPU through libpcaone_gb300.so; there is no CPU path.
"""
from __future__ import annotations

import os
from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import capi
from .synthetic import read_bed


class FileBed:
    """PLINK fileset on the GPU (src/FilePlink.hpp:7-47, FilePlink.cpp:26-120).

    ``memory`` (GB of device memory for the streamed blocks, the -m/--memory
    option, src/Cmd.cpp) selects the out-of-core form (FilePlink.cpp:122-218):
    the rows stay in pinned host memory and SNP blocks are streamed to the GPU;
    the window method's shuffle then follows permute_plink with ``buffer`` GB
    (the --buffer option) as the reference's out-of-core mode does.

    ``maf`` (the --maf option) keeps the SNPs whose minor allele frequency
    exceeds it (Data::filter_snps_resize_F, called by read_all at
    FilePlink.cpp:61); ``keepSNPs`` then lists their rows in the file.
    """

    def __init__(self, prefix: Optional[str] = None, *, packed: Optional[np.ndarray] = None,
                 nsamples: Optional[int] = None, device: int = 0, verbose: int = 0,
                 memory: Optional[float] = None, buffer: int = 2, maf: float = 0.0):
        self.ctx = capi.Context(device, verbose)
        self.out_of_core = memory is not None
        budget = int(memory * (1 << 30)) if memory is not None else 0
        if prefix is not None:
            fam = prefix + ".fam"
            bim = prefix + ".bim"
            with open(fam) as f:
                n = sum(1 for _ in f)
            with open(bim) as f:
                m = sum(1 for _ in f)
            with open(prefix + ".bed", "rb") as f:
                image = f.read()
            if self.out_of_core:
                self.ctx.load_bed_file_image_stream(image, m, n, budget, buffer)
            else:
                self.ctx.load_bed_file_image(image, m, n)
        elif packed is not None and nsamples is not None:
            if self.out_of_core:
                self.ctx.load_bed_stream(packed, nsamples, budget, buffer_gb=buffer)
            else:
                self.ctx.load_bed(packed, nsamples)
        else:
            raise ValueError("give a PLINK prefix or packed genotypes with nsamples")
        self._finish_read(maf)

    def _finish_read(self, maf: float):
        if maf > 0:
            self.ctx.filter_maf(maf)
        self.nsamples = self.ctx.nsamples
        self.nsnps = self.ctx.nsnps
        self.keepSNPs = self.ctx.kept_snps() if maf > 0 else np.empty(0, dtype=np.int64)
        self._counts = None

    @property
    def F(self) -> np.ndarray:
        return self.counts()[1]

    def counts(self):
        if self._counts is None:
            self._counts = self.ctx.counts()
        return self._counts

    def perform_op(self, x: np.ndarray, standardize: bool = True) -> np.ndarray:
        """ArnoldiOpData::perform_op (src/Arnoldi.cpp:18-46): y = X X^T x."""
        return self.ctx.matvec(x, standardize)

    def close(self):
        self.ctx.close()


class FilePgen(FileBed):
    """PLINK2 fileset on the GPU (src/FilePgen.hpp:13-40): the sample count from
    the .psam (lines not starting with '#'), hard calls from the .pgen (storage
    modes 0x01-0x04; variable-width files are decoded by pgenlib on the host and
    given as ``genovecs``, rows of 2-bit ALT counts with 3 = missing); ``maf``
    as for FileBed (FilePgen.cpp:53)."""

    def __init__(self, prefix: Optional[str] = None, *, genovecs: Optional[np.ndarray] = None,
                 nsamples: Optional[int] = None, device: int = 0, verbose: int = 0, maf: float = 0.0):
        self.ctx = capi.Context(device, verbose)
        self.out_of_core = False
        if prefix is not None:
            with open(prefix + ".psam") as f:
                n = sum(1 for line in f if line.strip() and not line.startswith("#"))
            with open(prefix + ".pgen", "rb") as f:
                image = f.read()
            self.ctx.load_pgen_file_image(image, n)
        elif genovecs is not None and nsamples is not None:
            self.ctx.load_pgen_genovecs(genovecs, nsamples)
        else:
            raise ValueError("give a PLINK2 prefix or hard calls with nsamples")
        self._finish_read(maf)


@dataclass
class Param:
    """The Param fields the RSVD path reads (src/Cmd.hpp:16-98) with the CLI's
    derived settings applied by ``finalize`` (src/Cmd.cpp:216, 228-232, 238)."""
    svd: int = 2
    k: int = 10
    oversamples: int = 10
    maxp: int = 20
    bands: int = 64
    seed: int = 112
    rand: int = 1
    emu: bool = False
    maxiter: int = 100
    tol: float = 1e-4
    tolem: float = 1e-5
    noshuffle: bool = False
    ploidy: int = 2
    precision: int = capi.PREC_BF16

    def finalize(self) -> "Param":
        self.oversamples = max(self.oversamples, self.k)
        if not self.emu:
            self.maxiter = 0
        return self

    def to_c(self, standardize: bool = True) -> capi.Params:
        return capi.default_params(svd=self.svd, k=self.k, oversamples=self.oversamples, maxp=self.maxp,
                                   bands=self.bands, seed=self.seed, rand=self.rand,
                                   perm=int(self.svd == 2 and not self.noshuffle), emu=int(self.emu),
                                   maxiter=self.maxiter, tol=self.tol, tolem=self.tolem, ploidy=self.ploidy,
                                   standardize=int(standardize), precision=self.precision)


class RsvdOpData:
    """RsvdOpData (src/Halko.hpp:6-42) backed by the GPU context of ``data``."""
    svd = 2

    def __init__(self, data: FileBed, k: int, os_: int = 10, *, params: Optional[Param] = None,
                 omega: Optional[np.ndarray] = None):
        self.data = data
        self.params = params or Param(svd=self.svd, k=k, oversamples=os_)
        self.params.svd = self.svd
        self.params.k, self.params.oversamples = k, os_
        if omega is not None:
            data.ctx.set_omega(omega)
        data.ctx.op_init(self.params.to_c())
        self.U = self.S = self.V = None

    def rows(self):
        return self.data.nsnps

    def cols(self):
        return self.data.nsamples

    def ranks(self):
        return self.params.k

    def oversamples(self):
        return self.params.oversamples

    def size(self):
        return self.ranks() + self.oversamples()

    def setFlags(self, update: bool, standardize: bool):  # noqa: N802 - reference name
        self.data.ctx.set_flags(update, standardize)

    def computeGandH(self, pi: int):  # noqa: N802
        return self.data.ctx.compute_g_and_h(pi)

    def computeUSV(self, p: int, tol: float):  # noqa: N802
        self.U, self.S, self.V, self.epochs = self.data.ctx.compute_usv(p, tol)
        return self


class NormalRsvdOpData(RsvdOpData):
    """Single-pass RSVD, -d 1 (src/Halko.hpp:44-66)."""
    svd = 1


class FancyRsvdOpData(RsvdOpData):
    """Window-based winSVD, -d 2 (src/Halko.hpp:68-93)."""
    svd = 2


def run_pca_with_halko(data: FileBed, params: Param, omega: Optional[np.ndarray] = None,
                       fileout: Optional[str] = None, printv: bool = True):
    """run_pca_with_halko (src/Halko.cpp:271-345): returns (U, S, V, em_iters);
    V rows are in the working SNP order, ``data.ctx.perm()`` maps them back.
    With ``fileout`` the text outputs are written as the reference writes them
    at the end of the run (write_eigs_files below)."""
    if omega is not None:
        data.ctx.set_omega(omega)
    U, S, V, it = data.ctx.run_halko(params.to_c())
    if fileout is not None:
        write_eigs_files(fileout, S, U, V, data.nsnps, data.ctx.perm(), printv=printv)
    return U, S, V, it


def _fmt(x: float) -> str:
    # a C++ stream at precision 6 in the default float field: printf's %.6g
    return f"{x:.6g}"


def _rows(A: np.ndarray) -> str:
    return "".join("\t".join(_fmt(x) for x in row) + "\n" for row in np.atleast_2d(A))


def write_eigs_files(fileout: str, S: np.ndarray, U: np.ndarray, V: Optional[np.ndarray], nsnps: int,
                     perm: Optional[np.ndarray] = None, printv: bool = True) -> None:
    """Data::write_eigs_files (src/Data.cpp:211-240) as run_pca_with_halko calls
    it (src/Halko.cpp:339): ``.sigvals`` (header ``#N,M``, then S), ``.eigvals``
    (S^2 / M), ``.eigvecs`` (U, N x k) and, with ``printv``, ``.loadings`` (V,
    M x k, rows back in the file's SNP order: working row i is SNP perm[i]);
    tab-separated, 6 significant digits.  The .mbim file (SNP metadata with
    allele frequencies) is left to the caller, which owns the .bim."""
    S = np.asarray(S, dtype=np.float64)
    U = np.asarray(U, dtype=np.float64)
    with open(fileout + ".sigvals", "w") as f:
        f.write(f"#{U.shape[0]},{nsnps if V is None else V.shape[0]}\n")
        f.write(_rows(S[:, None]))
    with open(fileout + ".eigvals", "w") as f:
        f.write(_rows((S ** 2 / nsnps)[:, None]))
    with open(fileout + ".eigvecs", "w") as f:
        f.write(_rows(U))
    if printv and V is not None:
        V = np.asarray(V, dtype=np.float64)
        if perm is not None and len(perm) == V.shape[0]:
            Vf = np.empty_like(V)
            Vf[np.asarray(perm, dtype=np.int64)] = V
            V = Vf
        with open(fileout + ".loadings", "w") as f:
            f.write(_rows(V))
