"""Shared helpers for the parity tests: golden fixtures and option parsing."""
from __future__ import annotations

import glob
import json
import os
from dataclasses import dataclass, field

import numpy as np

GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@dataclass
class RunOptions:
    """The PCAone options a case uses, with the CLI's derived settings applied
    (src/Cmd.cpp:216 oversamples >= k; :228-232 maxiter = 0 unless EM;
    :238 shuffle for -d 2 unless -S)."""
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
    scale: int = -9
    memory: float = 0.0  # -m GB: out-of-core (src/Cmd.cpp:218)
    maf: float = 0.0     # --maf: SNP filter before the run (src/Cmd.cpp:220)
    extra: dict = field(default_factory=dict)

    @property
    def perm(self) -> bool:
        return self.svd == 2 and not self.noshuffle

    @property
    def L(self) -> int:
        return self.k + self.oversamples


def parse_options(opts) -> RunOptions:
    o = RunOptions()
    it = iter(opts)
    for a in it:
        if a in ("-d", "--svd"):
            o.svd = int(next(it))
        elif a in ("-k", "--pc"):
            o.k = int(next(it))
        elif a == "--maxp":
            o.maxp = int(next(it))
        elif a in ("-w", "--batches"):
            o.bands = int(next(it))
        elif a == "--seed":
            o.seed = int(next(it))
        elif a == "--rand":
            o.rand = int(next(it))
        elif a == "--oversamples":
            o.oversamples = int(next(it))
        elif a == "--maxiter":
            o.maxiter = int(next(it))
        elif a == "--tol-rsvd":
            o.tol = float(next(it))
        elif a == "--tol-em":
            o.tolem = float(next(it))
        elif a in ("-S", "--no-shuffle"):
            o.noshuffle = True
        elif a == "--emu":
            o.emu = True
        elif a in ("-C", "--scale"):
            o.scale = int(next(it))
        elif a in ("-b", "-B", "-p", "--pgen"):
            next(it)
        elif a in ("-m", "--memory"):
            o.memory = float(next(it))
        elif a == "--maf":
            o.maf = float(next(it))
        else:
            raise ValueError(f"option {a} not handled")
    o.oversamples = max(o.oversamples, o.k)
    if not o.emu:
        o.maxiter = 0
    return o


@dataclass
class GoldenCase:
    name: str
    packed: np.ndarray
    nsamples: int
    nsnps: int
    opts: RunOptions
    ref: dict


def golden_cases(out_of_core: bool = False, maf: bool = False):
    """PLINK fixtures (packed genotypes): the in-core runs, with out_of_core
    the reference's -m runs, with maf the --maf runs (every row of the file in
    ``packed`` and nsnps; ref["keep"] the kept rows, ref["meta"][1] their
    number)."""
    out = []
    for path in sorted(glob.glob(os.path.join(GOLDEN_DIR, "*.npz"))):
        z = np.load(path)
        if "packed" not in z.files:
            continue
        opts = parse_options(json.loads(str(z["options"])))
        if (opts.memory > 0) != out_of_core or (opts.maf > 0) != maf:
            continue
        ref = {k: z[k] for k in z.files if k not in ("packed", "options")}
        meta = ref["meta"]
        packed = z["packed"]
        out.append(GoldenCase(os.path.basename(path)[:-4], packed, int(meta[0]), int(packed.shape[0]), opts, ref))
    return out


@dataclass
class BinaryCase:
    name: str
    dense: np.ndarray        # M x N float16 values (read by the reference as float32)
    nsamples: int
    nsnps: int
    opts: RunOptions
    ref: dict


def binary_cases():
    """FileBinary fixtures (dense float16 dosages, -B ... -C 0)."""
    out = []
    for path in sorted(glob.glob(os.path.join(GOLDEN_DIR, "*.npz"))):
        z = np.load(path)
        if "dense" not in z.files:
            continue
        opts = parse_options(json.loads(str(z["options"])))
        ref = {k: z[k] for k in z.files if k not in ("dense", "options")}
        meta = ref["meta"]
        out.append(BinaryCase(os.path.basename(path)[:-4], z["dense"], int(meta[0]), int(meta[1]), opts, ref))
    return out


def pgen_cases():
    """PLINK2 fixtures: fixed-width .pgen hard calls (genovec rows), read by the
    reference through its pgenlib (-p)."""
    out = []
    for path in sorted(glob.glob(os.path.join(GOLDEN_DIR, "*.npz"))):
        z = np.load(path)
        if "genovec" not in z.files:
            continue
        opts = parse_options(json.loads(str(z["options"])))
        ref = {k: z[k] for k in z.files if k not in ("genovec", "options")}
        meta = ref["meta"]
        out.append(GoldenCase(os.path.basename(path)[:-4], z["genovec"], int(meta[0]), int(meta[1]), opts, ref))
    return out


def pgen_image(genovec: np.ndarray, nsamples: int) -> bytes:
    """A fixed-width (storage mode 0x02) .pgen of the genovec rows: magic, mode,
    variant count, sample count, control byte, then the records."""
    m = genovec.shape[0]
    head = bytes([0x6C, 0x1B, 0x02]) + int(m).to_bytes(4, "little") + int(nsamples).to_bytes(4, "little") + bytes([0])
    return head + np.ascontiguousarray(genovec[:, : (nsamples + 3) // 4]).tobytes()


def golden_case(name: str) -> GoldenCase:
    for c in golden_cases() + golden_cases(out_of_core=True) + golden_cases(maf=True):
        if c.name == name:
            return c
    raise KeyError(name)


def align_signs(A: np.ndarray, B: np.ndarray) -> np.ndarray:
    """Columns of A with their signs matched to B's (singular vectors are
    determined up to sign)."""
    s = np.sign(np.sum(A * B, axis=0))
    s[s == 0] = 1.0
    return A * s[None, :]
