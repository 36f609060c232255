"""Flux input (InputIsDeltaFlux 0): the reader turns flux into delta_F before
it masks outliers, with the spectrum's own mean flux (UseChunksMeanFlux 1) or
with F-bar(z) from a MeanFluxFile (conv::, core/fiducial_cosmology.cpp:33-169;
core/one_qso_estimate.cpp:62-65).

The tiny workload's spectra are written as flux F = F-bar(z) (1 + delta) with
noise F-bar(z) sigma; the compiled reference reads them with each option, and
its chunks (lambda / LYA_REST, delta, ivar) are the checker for both the
restatement's reader and the C++ facade's (OneQSOEstimate::readQsoFile,
tests/cpp/read_spectra.cpp).  The mean-flux table covers z 2.15-2.65, inside
the data, so both of its linear continuations are used.  Host-only.
"""
import os
import shutil
import struct
import subprocess

import numpy as np
import pytest

from oracle import qmle_port as P
from oracle import refdump

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LYA = 1215.67


def _fbar(z):
    return np.exp(-0.0023 * (1.0 + z) ** 3.65)


def _flux_workload():
    from lyspeq_gb300 import synth
    w = synth.make_workload("tiny")
    for s in w.spectra:
        fb = _fbar(np.asarray(s.wave) / LYA - 1.0)
        s.delta = fb * (1.0 + np.asarray(s.delta))
        s.sigma = fb * np.asarray(s.sigma)
    return w


def _reference_chunks(w, tmp_path, mode, mf_path):
    from lyspeq_gb300 import synth
    cfg = synth.write_reference_inputs(w, str(tmp_path))
    text = open(cfg).read()
    assert "InputIsDeltaFlux 1\n" in text
    keys = "UseChunksMeanFlux 1\n" if mode == "mean" else f"MeanFluxFile {mf_path}\n"
    open(cfg, "w").write(text.replace("InputIsDeltaFlux 1\n", "InputIsDeltaFlux 0\n" + keys))
    dump = refdump.run_driver(cfg, str(tmp_path / "dump.bin"))
    assert dump.chunks
    return {(float(c.wave[0]), len(c.wave)): c for c in dump.chunks}, cfg


@pytest.mark.skipif(not refdump.available(), reason="compiled reference not built")
@pytest.mark.parametrize("mode", ["mean", "file"])
def test_flux_input_matches_the_reference(tmp_path, mode):
    w = _flux_workload()
    zt = np.linspace(2.15, 2.65, 11)
    mf_path = tmp_path / "meanflux.bin"
    with open(mf_path, "wb") as f:
        f.write(struct.pack("<i", len(zt)))
        f.write(zt.astype("<f8").tobytes())
        f.write(_fbar(zt).astype("<f8").tobytes())
    ref, cfg = _reference_chunks(w, tmp_path, mode, mf_path)
    # the restatement
    s = P.Settings(max_forest_length=w.max_forest_length, cont_logl_order=w.cont_logl_order,
                   cont_l_order=w.cont_l_order, input_is_delta_flux=False,
                   use_chunks_mean_flux=mode == "mean", mean_flux=(zt, _fbar(zt)) if mode == "file" else None)
    mine = P.chunks_from_spectra(w.spectra, w.bins, w.table_index(), s)
    assert len(mine) == len(ref)
    tol = 0.0 if mode == "mean" else 1e-13
    for ch in mine:
        c = ref[(float(ch.wave[0]), len(ch.wave))]
        assert np.array_equal(ch.wave, c.wave)
        assert np.max(np.abs(ch.delta - c.delta)) <= tol * np.max(np.abs(c.delta))
        assert np.max(np.abs(ch.ivar - c.ivar)) <= tol * np.max(np.abs(c.ivar))
    # the facade
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path / "read_spectra")
    subprocess.run([gxx, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(HERE, "cpp", "read_spectra.cpp"), "-o", exe], check=True)
    spec_dir = os.path.dirname(cfg)
    files = sorted(os.path.join(dp, f) for dp, _, fs in os.walk(spec_dir) for f in fs if f.endswith(".dat"))
    assert len(files) == len(w.spectra)
    out = tmp_path / "facade.bin"
    zlo = w.bins.z_centers[0] - w.bins.dz / 2
    zhi = w.bins.z_centers[-1] + w.bins.dz / 2
    subprocess.run([exe, str(out), "1" if mode == "mean" else "2", str(mf_path) if mode == "file" else "-",
                    repr(float(zlo)), repr(float(zhi)), repr(float(w.max_forest_length)), "1"] + files, check=True)
    buf, pos = open(out, "rb").read(), 0
    got = {}
    for _ in files:
        (nch,), pos = struct.unpack_from("<q", buf, pos), pos + 8
        for _ in range(max(nch, 0)):
            (n,), pos = struct.unpack_from("<q", buf, pos), pos + 8
            if n == 0:
                continue
            arr = np.frombuffer(buf, "<f8", 3 * n, pos).reshape(3, n)
            pos += 24 * n
            wave = arr[0] / LYA
            got[(float(wave[0]), n)] = (wave, arr[1], arr[2])
    assert pos == len(buf)
    for key, c in ref.items():
        wave, delta, ivar = got[key]
        assert np.array_equal(wave, c.wave)
        assert np.max(np.abs(delta - c.delta)) <= tol * np.max(np.abs(c.delta))
        assert np.max(np.abs(ivar - c.ivar)) <= tol * np.max(np.abs(c.ivar))
