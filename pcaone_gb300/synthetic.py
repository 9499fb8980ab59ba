"""Seeded synthetic PLINK genotypes (Balding-Nichols populations).

The workloads are described by sizes and population-genetic parameters only;
no public dataset is used.  Generation is split in two halves:

* ``draw_population_model`` (host, numpy ``default_rng``): ancestral allele
  frequencies, Balding-Nichols population frequencies
  ``Beta(p(1-F)/F, (1-p)(1-F)/F)``, per-sample ancestry weights (one-hot for
  unadmixed samples, Dirichlet for admixed ones) and per-sample / per-SNP
  missing rates.
* genotype sampling, which is a pure function of (seed, SNP index, sample
  index) through a counter-based SplitMix64 hash.  ``sample_packed_bed`` below
  is the numpy form; the CUDA library carries the same arithmetic
  (``pcaone_gpu_load_synthetic``) for workloads too large to draw on the host, and
  both produce identical bytes.

PLINK .bed coding of one genotype (2 bits, little-endian inside each byte,
sample ``i`` of a SNP at bits ``2*(i % 4)`` of byte ``i // 4``):
``00`` two copies of A1, ``10`` one copy, ``11`` none, ``01`` missing, as read
by the reference in ``src/Common.hpp:50-59``.  Padding bits of the last byte
of a SNP are written as zero unless ``pad_garbage`` is set.
"""
from __future__ import annotations

import dataclasses
import os
from typing import Optional, Sequence

import numpy as np

_MASK64 = np.uint64(0xFFFFFFFFFFFFFFFF)
_GAMMA = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)

# stream keys of the three independent uniforms drawn per genotype
KEY_ALLELE_A = 0x243F6A8885A308D3
KEY_ALLELE_B = 0x13198A2E03707344
KEY_MISSING = 0xA4093822299F31D0


def mix64(x: np.ndarray) -> np.ndarray:
    """SplitMix64 output function (Steele, Lea & Flood 2014) on uint64 arrays."""
    with np.errstate(over="ignore"):
        z = (x + _GAMMA) & _MASK64
        z = ((z ^ (z >> np.uint64(30))) * _M1) & _MASK64
        z = ((z ^ (z >> np.uint64(27))) * _M2) & _MASK64
        return z ^ (z >> np.uint64(31))


def uniform01(seed: int, key: int, counter: np.ndarray) -> np.ndarray:
    """Uniform double in [0,1) from the top 53 bits of mix64(counter ^ stream)."""
    stream = mix64(np.array([(seed * 0x2545F4914F6CDD1D + key) & 0xFFFFFFFFFFFFFFFF],
                            dtype=np.uint64))[0]
    h = mix64(counter ^ stream)
    return (h >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


@dataclasses.dataclass
class PopulationModel:
    """Per-SNP population frequencies and per-sample weights / missing rates."""
    seed: int
    nsamples: int
    nsnps: int
    freq: np.ndarray          # (M, npop) float64: A1 frequency per SNP and population
    weights: np.ndarray       # (N, npop) float64: ancestry proportions per sample
    miss_sample: np.ndarray   # (N,) float64
    miss_snp: np.ndarray      # (M,) float64
    pop_of_sample: np.ndarray  # (N,) int32, -1 for admixed samples

    @property
    def npop(self) -> int:
        return self.freq.shape[1]


def draw_population_model(nsamples: int, nsnps: int, npop: int, fst: Sequence[float] | float,
                          seed: int = 1, anc: str = "uniform", anc_range=(0.05, 0.5),
                          admixed_frac: float = 0.0, dirichlet_alpha: float = 0.5,
                          mcar: float = 0.0, miss_sample_beta: Optional[tuple] = None,
                          miss_snp_beta: Optional[tuple] = None) -> PopulationModel:
    rng = np.random.default_rng(seed)
    fst_arr = np.broadcast_to(np.asarray(fst, dtype=np.float64), (npop,)).copy()
    if anc == "uniform":
        p = rng.uniform(anc_range[0], anc_range[1], size=nsnps)
    elif anc == "beta":
        # Beta(0.5,0.5) truncated to anc_range by redrawing out-of-range values
        p = rng.beta(0.5, 0.5, size=nsnps)
        bad = (p < anc_range[0]) | (p > anc_range[1])
        while bad.any():
            p[bad] = rng.beta(0.5, 0.5, size=int(bad.sum()))
            bad = (p < anc_range[0]) | (p > anc_range[1])
    else:
        raise ValueError(f"unknown ancestral distribution {anc!r}")
    freq = np.empty((nsnps, npop), dtype=np.float64)
    for k in range(npop):
        f = fst_arr[k]
        a = p * (1.0 - f) / f
        b = (1.0 - p) * (1.0 - f) / f
        freq[:, k] = rng.beta(a, b)
    n_adm = int(round(admixed_frac * nsamples))
    n_pure = nsamples - n_adm
    pop = (np.arange(n_pure, dtype=np.int64) * npop) // max(n_pure, 1)
    weights = np.zeros((nsamples, npop), dtype=np.float64)
    weights[np.arange(n_pure), pop] = 1.0
    pop_of_sample = np.full(nsamples, -1, dtype=np.int32)
    pop_of_sample[:n_pure] = pop
    if n_adm:
        weights[n_pure:] = rng.dirichlet(np.full(npop, dirichlet_alpha), size=n_adm)
    if miss_sample_beta is not None:
        miss_sample = rng.beta(*miss_sample_beta, size=nsamples)
    else:
        miss_sample = np.full(nsamples, float(mcar))
    if miss_snp_beta is not None:
        miss_snp = rng.beta(*miss_snp_beta, size=nsnps)
    else:
        miss_snp = np.zeros(nsnps)
    return PopulationModel(seed, nsamples, nsnps, freq, weights, miss_sample, miss_snp,
                           pop_of_sample)


def bytes_per_snp(nsamples: int) -> int:
    """Packed .bed bytes per SNP, ``(N+3)>>2`` as in src/FilePlink.hpp:19."""
    return (nsamples + 3) >> 2


def sample_codes(model: PopulationModel, snp_lo: int, snp_hi: int) -> np.ndarray:
    """2-bit PLINK codes (uint8 in 0..3) of SNPs [snp_lo, snp_hi) x all samples.

    Per genotype: p = sum_k w_ik * freq_jk (sequential sum, round-to-nearest, no
    fused multiply-add), r = 1 - (1 - a_i) * (1 - b_j); missing if u_m < r,
    else dosage = [u_a < p] + [u_b < p].
    """
    n = model.nsamples
    j = np.arange(snp_lo, snp_hi, dtype=np.uint64)[:, None]
    i = np.arange(n, dtype=np.uint64)[None, :]
    counter = (j << np.uint64(32)) | i
    fr = model.freq[snp_lo:snp_hi]                     # (m, npop)
    p = np.zeros((snp_hi - snp_lo, n), dtype=np.float64)
    for k in range(model.npop):
        p = p + model.weights[None, :, k] * fr[:, k:k + 1]
    r = 1.0 - (1.0 - model.miss_sample[None, :]) * (1.0 - model.miss_snp[snp_lo:snp_hi, None])
    ua = uniform01(model.seed, KEY_ALLELE_A, counter)
    ub = uniform01(model.seed, KEY_ALLELE_B, counter)
    um = uniform01(model.seed, KEY_MISSING, counter)
    dosage = (ua < p).astype(np.uint8) + (ub < p).astype(np.uint8)
    code = np.where(dosage == 2, 0, np.where(dosage == 1, 2, 3)).astype(np.uint8)
    code[um < r] = 1
    return code


KEY_DOSAGE_NOISE = 0xD05E


def sample_dosages(model: PopulationModel, sd: float = 0.1, snp_lo: int = 0, snp_hi: Optional[int] = None,
                   ) -> np.ndarray:
    """Continuous dosages of SNPs [snp_lo, snp_hi) x all samples (float16,
    M' x N): the sampled allele count d in {0, 1, 2} (missing genotypes of the
    model are drawn as observed) plus Gaussian noise of standard deviation sd
    (Box-Muller on two hashed uniforms), clipped to [0, 2] and rounded to
    float16, the storage of imputed dosages."""
    snp_hi = model.nsnps if snp_hi is None else snp_hi
    code = sample_codes(model, snp_lo, snp_hi)
    n = model.nsamples
    j = np.arange(snp_lo, snp_hi, dtype=np.uint64)[:, None]
    i = np.arange(n, dtype=np.uint64)[None, :]
    counter = (j << np.uint64(32)) | i
    # allele counts without the missing draw: recompute from the two allele draws
    fr = model.freq[snp_lo:snp_hi]
    p = np.zeros((snp_hi - snp_lo, n), dtype=np.float64)
    for k in range(model.npop):
        p = p + model.weights[None, :, k] * fr[:, k:k + 1]
    ua = uniform01(model.seed, KEY_ALLELE_A, counter)
    ub = uniform01(model.seed, KEY_ALLELE_B, counter)
    d = (ua < p).astype(np.float64) + (ub < p).astype(np.float64)
    u1 = uniform01(model.seed, KEY_DOSAGE_NOISE, counter)
    u2 = uniform01(model.seed, KEY_DOSAGE_NOISE + 1, counter)
    z = np.sqrt(-2.0 * np.log(np.maximum(u1, 1e-300))) * np.cos(2.0 * np.pi * u2)
    del code
    return np.clip(d + sd * z, 0.0, 2.0).astype(np.float16)


def write_binary(path: str, values: np.ndarray) -> None:
    """The reference's FileBinary format (src/FileBinary.hpp:17-18,
    src/FileBinary.cpp:21-46): uint32 SNPs, uint32 samples, then float32
    values SNP by SNP."""
    v = np.ascontiguousarray(values, dtype=np.float32)
    with open(path, "wb") as f:
        f.write(np.array([v.shape[0], v.shape[1]], dtype=np.uint32).tobytes())
        f.write(v.tobytes())


def read_binary(path: str) -> np.ndarray:
    with open(path, "rb") as f:
        m, n = np.frombuffer(f.read(8), dtype=np.uint32)
        return np.frombuffer(f.read(), dtype=np.float32).reshape(int(m), int(n))


def pack_codes(code: np.ndarray, pad_garbage: bool = False, seed: int = 0) -> np.ndarray:
    """Pack (m, N) 2-bit codes into (m, ceil(N/4)) bytes, PLINK SNP-major order."""
    m, n = code.shape
    nb = bytes_per_snp(n)
    padded = np.zeros((m, nb * 4), dtype=np.uint8)
    padded[:, :n] = code
    if pad_garbage and nb * 4 > n:
        rng = np.random.default_rng(seed + 77)
        padded[:, n:] = rng.integers(0, 4, size=(m, nb * 4 - n), dtype=np.uint8)
    q = padded.reshape(m, nb, 4)
    return (q[:, :, 0] | (q[:, :, 1] << 2) | (q[:, :, 2] << 4) | (q[:, :, 3] << 6)).astype(np.uint8)


def sample_packed_bed(model: PopulationModel, chunk: int = 4096, pad_garbage: bool = False) -> np.ndarray:
    """Packed genotype matrix (M, ceil(N/4)) uint8 for the whole model (numpy path)."""
    out = np.empty((model.nsnps, bytes_per_snp(model.nsamples)), dtype=np.uint8)
    for lo in range(0, model.nsnps, chunk):
        hi = min(model.nsnps, lo + chunk)
        out[lo:hi] = pack_codes(sample_codes(model, lo, hi), pad_garbage, model.seed + lo)
    return out


BED_MAGIC = bytes([0x6C, 0x1B, 0x01])


def write_plink(prefix: str, packed: np.ndarray, nsamples: int) -> None:
    """Write prefix.bed/.bim/.fam (only line counts of .bim/.fam are read downstream)."""
    m = packed.shape[0]
    with open(prefix + ".bed", "wb") as f:
        f.write(BED_MAGIC)
        f.write(np.ascontiguousarray(packed).tobytes())
    with open(prefix + ".bim", "w") as f:
        f.write("".join(f"1\tsnp{j}\t0\t{j + 1}\tA\tG\n" for j in range(m)))
    with open(prefix + ".fam", "w") as f:
        f.write("".join(f"fam{i}\tind{i}\t0\t0\t0\t-9\n" for i in range(nsamples)))


def read_bed(prefix: str, nsamples: Optional[int] = None, nsnps: Optional[int] = None) -> tuple:
    """Read prefix.bed into (packed (M, ceil(N/4)) uint8, N, M).

    N and M come from the .fam/.bim line counts when not given, as in
    src/FilePlink.hpp:13-19; the magic bytes are checked as in
    src/FilePlink.hpp:24-27.
    """
    if nsamples is None:
        with open(prefix + ".fam") as f:
            nsamples = sum(1 for _ in f)
    if nsnps is None:
        with open(prefix + ".bim") as f:
            nsnps = sum(1 for _ in f)
    nb = bytes_per_snp(nsamples)
    with open(prefix + ".bed", "rb") as f:
        head = f.read(3)
        if head != BED_MAGIC:
            raise ValueError("Incorrect magic number in plink bed file.")
        data = np.fromfile(f, dtype=np.uint8, count=nb * nsnps)
    if data.size != nb * nsnps:
        raise ValueError(f"truncated .bed: expected {nb * nsnps} bytes, found {data.size}")
    return data.reshape(nsnps, nb), nsamples, nsnps


# Workloads: sizes and population-genetic parameters of the five configurations.
WORKLOADS = {
    "c1": dict(nsamples=2000, nsnps=20000, npop=3, fst=0.05, anc="uniform", anc_range=(0.05, 0.5),
               mcar=0.01, k=10, p=10, maxp=6, bands=64),
    "c2": dict(nsamples=100_000, nsnps=500_000, npop=5, fst=[0.01, 0.02, 0.05, 0.1, 0.2],
               anc="uniform", anc_range=(0.01, 0.5), mcar=0.005, k=20, p=20, maxp=6, bands=64),
    "c3": dict(nsamples=200_000, nsnps=1_000_000, npop=8, fst=0.05, anc="beta", anc_range=(0.01, 0.99),
               admixed_frac=0.02, mcar=0.0, k=40, p=10, maxp=6, bands=64),
    # scaled-down c2 (0.5 GB packed, still larger than L2) for profiling captures
    "c2s": dict(nsamples=20_000, nsnps=100_000, npop=5, fst=[0.01, 0.02, 0.05, 0.1, 0.2],
                anc="uniform", anc_range=(0.01, 0.5), mcar=0.005, k=20, p=20, maxp=6, bands=64),
    # the c2 window shape (7,812 SNPs x 100,000 samples) with 1/8 of the SNPs
    # (1.56 GB packed) for profiling captures of single window launches
    "c2p": dict(nsamples=100_000, nsnps=62_500, npop=5, fst=[0.01, 0.02, 0.05, 0.1, 0.2],
                anc="uniform", anc_range=(0.01, 0.5), mcar=0.005, k=20, p=20, maxp=6, bands=8),
    # the c3 window shape (15,625 SNPs x 200,000 samples, k=40, p=10) as one
    # single-pass window (0.78 GB packed) for profiling captures of single launches
    "c3p": dict(nsamples=200_000, nsnps=15_625, npop=8, fst=0.05, anc="beta", anc_range=(0.01, 0.99),
                admixed_frac=0.02, mcar=0.0, k=40, p=10, maxp=6, bands=64, svd=1, perm=0),
    # continuous dosages held as FP16 (FileBinary input, -C 0): c5 is 1M SNPs x 100k
    # samples (200 GB FP16, run without the shuffle: a shuffled copy would not
    # fit), c5s the same model at 100k SNPs (20 GB)
    "c5": dict(nsamples=100_000, nsnps=1_000_000, npop=6, fst=[0.01, 0.02, 0.04, 0.06, 0.1, 0.15],
               anc="uniform", anc_range=(0.05, 0.5), k=20, p=20, maxp=6, bands=64, dense=True, sd=0.1, perm=0),
    "c5s": dict(nsamples=100_000, nsnps=100_000, npop=6, fst=[0.01, 0.02, 0.04, 0.06, 0.1, 0.15],
                anc="uniform", anc_range=(0.05, 0.5), k=20, p=20, maxp=6, bands=64, dense=True, sd=0.1),
    # EM imputation (-d 2 -S: no shuffle, the reference's shuffled EMU path has a defect)
    "c4": dict(nsamples=50_000, nsnps=300_000, npop=4, fst=0.05, anc="uniform", anc_range=(0.05, 0.5),
               miss_sample_beta=(1, 20), miss_snp_beta=(1, 50), k=10, p=10, maxp=6, bands=64,
               emu=True, tolem=1e-6, maxiter=100, perm=0),
}


def model_for(name: str, seed: int = 1, **override) -> PopulationModel:
    cfg = dict(WORKLOADS[name])
    cfg.update(override)
    keys = ("nsamples", "nsnps", "npop", "fst", "anc", "anc_range", "admixed_frac", "mcar",
            "miss_sample_beta", "miss_snp_beta")
    return draw_population_model(seed=seed, **{k: cfg[k] for k in keys if k in cfg})


if __name__ == "__main__":  # pragma: no cover - convenience CLI
    import argparse
    ap = argparse.ArgumentParser(description="write a synthetic PLINK fileset")
    ap.add_argument("prefix")
    ap.add_argument("--workload", default="c1")
    ap.add_argument("--nsamples", type=int)
    ap.add_argument("--nsnps", type=int)
    ap.add_argument("--seed", type=int, default=1)
    a = ap.parse_args()
    ov = {k: v for k, v in (("nsamples", a.nsamples), ("nsnps", a.nsnps)) if v}
    mdl = model_for(a.workload, a.seed, **ov)
    os.makedirs(os.path.dirname(os.path.abspath(a.prefix)), exist_ok=True)
    write_plink(a.prefix, sample_packed_bed(mdl), mdl.nsamples)
