"""Reader for the oracle driver's dump (test infrastructure only).

The dump is written by ``oracle/refbuild/chunk_driver.cpp``, which runs
lyspeq's own ``Chunk::oneQSOiteration`` (core/chunk_estimate.cpp:837-914) on
every chunk of a config and then the global Newton-Raphson step
(core/quadratic_estimate.cpp:456-457, 261-318).  Layout: little-endian,
``LQGREF02`` magic, four int32 (nkz, nk, nz, nchunks), one record per chunk
(with the chunk's resolution matrix when the driver ran with ``--reso``),
then a ``GLOBAL01`` block.
"""
from __future__ import annotations

import dataclasses
import os
import subprocess
import sys

import numpy as np

from oracle.refsrc import reference_root

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
DRIVER = os.path.join(REF_DIR, "chunk_driver")
DRIVER_FOPT = os.path.join(REF_DIR, "chunk_driver_fopt")   # built with -DFISHER_OPTIMIZATION
LYAPOWER = os.path.join(REF_DIR, "LyaPowerEstimate")
REFERENCE_PY = os.path.join(reference_root(), "py")   # lyspeq's own helper scripts (smoothing)


@dataclasses.dataclass
class RefChunk:
    qso: int
    index: int
    n: int
    fisher_index_start: int
    nq: int
    kbin_upp: int
    r_fwhm: int
    status: int
    dv: float
    wave: np.ndarray | None   # lambda / LYA_REST (= 1 + z), as the chunk holds it
    delta: np.ndarray | None
    ivar: np.ndarray | None
    d: np.ndarray
    b: np.ndarray
    t: np.ndarray
    fisher: np.ndarray        # nq x nq, upper triangle filled, not halved
    rmat: np.ndarray | None = None   # values[ndiags][n] (diagonal) or rows[n][nelem]
    rmat_dia: bool = False


@dataclasses.dataclass
class RefDump:
    nkz: int
    nk: int
    nz: int
    chunks: list
    fisher: np.ndarray        # global, halved and symmetrised
    dbt: np.ndarray           # 3 x nkz sums before Fisher weighting
    solver_invfisher: np.ndarray
    inverse_fisher: np.ndarray
    theta: np.ndarray
    damped: int
    dof: int
    damp: float
    pfid: np.ndarray
    t_chunks: float
    t_global: float
    boot_mean: np.ndarray | None = None        # FastBootstrap: mean of the realizations
    boot_cov: np.ndarray | None = None         # F^-1 (cov / 4) F^-T
    boot_real: np.ndarray | None = None        # realizations [nboots][nkz]
    n_qso: int = 0
    boot_complete: bool = False                # FastBootstrap 0: boot_cov is the covariance itself
    boot_valid: int = 0                        # realizations whose Fisher solve succeeded


class _Reader:
    def __init__(self, buf: bytes):
        self.buf = buf
        self.pos = 0

    def i(self, n=1):
        v = np.frombuffer(self.buf, dtype="<i4", count=n, offset=self.pos)
        self.pos += 4 * n
        return int(v[0]) if n == 1 else v.copy()

    def d(self, n):
        v = np.frombuffer(self.buf, dtype="<f8", count=n, offset=self.pos)
        self.pos += 8 * n
        return v.copy()

    def magic(self, want: bytes):
        got = self.buf[self.pos:self.pos + 8]
        if got != want:
            raise ValueError(f"bad dump: expected {want!r}, got {got!r}")
        self.pos += 8


def read_dump(path: str) -> RefDump:
    with open(path, "rb") as f:
        r = _Reader(f.read())
    r.magic(b"LQGREF02")
    nkz, nk, nz, nch = (r.i() for _ in range(4))
    chunks = []
    for _ in range(nch):
        qso, idx, n, fis, nq, kup, rf, st = (r.i() for _ in range(8))
        dv = float(r.d(1)[0])
        has_pix = r.i()
        w = dl = iv = None
        if has_pix:
            w, dl, iv = r.d(n), r.d(n), r.d(n)
        nrm, rdia, nelem = r.i(), r.i(), r.i()
        rm = None
        if nrm:
            rm = r.d(nrm)
            rm = rm.reshape(nelem, n) if rdia else rm.reshape(n, nelem)
        d, b, t = r.d(nq), r.d(nq), r.d(nq)
        fm = r.d(nq * nq).reshape(nq, nq)
        chunks.append(RefChunk(qso, idx, n, fis, nq, kup, rf, st, dv, w, dl, iv, d, b, t, fm,
                               rm, bool(rdia)))
    r.magic(b"GLOBAL01")
    fisher = r.d(nkz * nkz).reshape(nkz, nkz)
    dbt = np.stack([r.d(nkz) for _ in range(3)])
    solver = r.d(nkz * nkz).reshape(nkz, nkz)
    invf = r.d(nkz * nkz).reshape(nkz, nkz)
    theta = r.d(nkz)
    damped, dof = r.i(), r.i()
    damp = float(r.d(1)[0])
    pfid = r.d(nkz)
    t_chunks, t_global = float(r.d(1)[0]), float(r.d(1)[0])
    dump = RefDump(nkz, nk, nz, chunks, fisher, dbt, solver, invf, theta, damped, dof, damp,
                   pfid, t_chunks, t_global)
    if r.pos < len(r.buf):
        complete = r.buf[r.pos:r.pos + 8] == b"BOOT0002"
        r.magic(b"BOOT0002" if complete else b"BOOT0001")
        nb, nq = r.i(), r.i()
        dump.n_qso = nq
        dump.boot_complete = complete
        dump.boot_valid = r.i() if complete else nb
        dump.boot_mean = r.d(nkz)
        dump.boot_cov = r.d(nkz * nkz).reshape(nkz, nkz)
        dump.boot_real = r.d(nb * nkz).reshape(nb, nkz)
    return dump


def available() -> bool:
    return os.path.exists(DRIVER)


@dataclasses.dataclass
class RefIteration:
    """Final state of lyspeq's OneDQuadraticPowerEstimate after iterate()."""
    theta: np.ndarray            # current_power_estimate_vector
    previous: np.ndarray         # previous_power_estimate_vector
    fits: np.ndarray             # powerspectra_fits (smoothed theta fed to the last iteration)
    fisher: np.ndarray           # fisher_matrix_sum, halved and symmetric
    inverse: np.ndarray          # inverse_fisher_matrix_sum
    dbt: np.ndarray              # 3 x nkz


def read_iteration(path: str) -> RefIteration:
    with open(path, "rb") as f:
        r = _Reader(f.read())
    r.magic(b"ITER0001")
    nkz = r.i()
    th, prev, fits = r.d(nkz), r.d(nkz), r.d(nkz)
    fm = r.d(nkz * nkz).reshape(nkz, nkz)
    inv = r.d(nkz * nkz).reshape(nkz, nkz)
    dbt = np.stack([r.d(nkz) for _ in range(3)])
    return RefIteration(th, prev, fits, fm, inv, dbt)


def run_driver(config: str, out: str, pixels: bool = True, threads: int | None = None,
               reso: bool = False, boots: int = 0, iterate: bool = False,
               boot_complete: bool = False, fisher_optimization: bool = False) -> RefDump:
    env = dict(os.environ)
    env.setdefault("OPENBLAS_NUM_THREADS", "1")
    # One OpenMP thread: with more, Chunk::_applyRedshiftInterp races on the
    # shared `low`/`tmp` bounds (core/chunk_estimate.cpp:486, 512-516) and the
    # redshift weights of some rows come out wrong from run to run.
    env["OMP_NUM_THREADS"] = str(threads or 1)
    args = [DRIVER_FOPT if fisher_optimization else DRIVER, config, out] + ([] if pixels else ["--no-pixels"]) + (["--reso"] if reso else []) \
        + (["--boot", str(boots)] if boots else []) + (["--boot-complete"] if boot_complete else []) \
        + (["--iterate"] if iterate else [])
    if iterate:
        # lyspeq's smoothing step runs its script smbivspline.py from PATH
        wrap = os.path.join(os.path.dirname(os.path.abspath(out)), "bin")
        os.makedirs(wrap, exist_ok=True)
        script = os.path.join(wrap, "smbivspline.py")
        with open(script, "w") as f:
            f.write(f"#!/bin/sh\nexec {sys.executable} {REFERENCE_PY}/smbivspline.py \"$@\"\n")
        os.chmod(script, 0o755)
        env["PATH"] = wrap + os.pathsep + env.get("PATH", "")
    subprocess.run(args, check=True, env=env, stdout=subprocess.DEVNULL,
                   stderr=subprocess.DEVNULL)
    return read_dump(out)
