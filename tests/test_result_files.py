"""The C++ facade's result files against lyspeq's own (host-only).

lyspeq writes, per iteration, the detailed estimate and the Fisher, inverse
Fisher and solver matrices (core/quadratic_estimate.cpp:616-751, 797-830).
The compiled reference's LyaPowerEstimate runs the small workload (64
spectra, 36 of them outside the redshift bins); its numbers are then
written again by the facade's writers (tests/cpp/write_outputs.cpp), which
count the spectra per redshift bin from the files themselves.  The matrix
files must come out byte for byte, every line of the detailed file a reader
parses the same (the data lines of its header included), except two columns
the writer recomputes from the printed numbers (Pest = Pfid + ThetaP, ErrorP =
sqrt of the inverse Fisher diagonal), which agree to the printing of their
inputs.  The
facade's PD13 fiducial power reproduces the Pfid column.
"""
import os
import shutil
import struct
import subprocess

import numpy as np
import pytest

from oracle import refdump

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SUFFIXES = ("_quadratic_power_estimate_detailed.txt", "_fisher_matrix.txt", "_inversefisher_matrix.txt",
            "_solver_invfishermatrix.txt")


def _matrix(path):
    return np.loadtxt(path, skiprows=1, ndmin=2)


@pytest.mark.skipif(not os.path.exists(refdump.LYAPOWER), reason="compiled reference not built")
def test_result_files_match_lyspeqs(tmp_path):
    from lyspeq_gb300 import synth
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    w = synth.make_workload("small")
    ref_dir = tmp_path / "ref"
    cfg = synth.write_reference_inputs(w, str(ref_dir))
    env = dict(os.environ, OMP_NUM_THREADS="1", OPENBLAS_NUM_THREADS="1")
    subprocess.run([refdump.LYAPOWER, cfg], check=True, env=env, stdout=subprocess.DEVNULL,
                   stderr=subprocess.DEVNULL)
    ref = {s: str(ref_dir / ("qmle_it1" + s)) for s in SUFFIXES}
    for p in ref.values():
        assert os.path.exists(p), p
    lines = open(ref[SUFFIXES[0]]).read().split("\n")
    data_comments = [ln for ln in lines if ln.startswith("# Damped") or ln.startswith("# Damping constant")]
    i = next(k for k, ln in enumerate(lines) if ln.startswith("# Damping constant"))
    data_comments += lines[i + 1:i + 3]          # "# Nz Nk" and the z-bin counts
    body = [ln for ln in lines if ln and not ln.startswith("#")]
    table = np.array([[float(x) for x in ln.split()] for ln in body[1:]])
    nkz = w.bins.nk * w.bins.nz
    assert table.shape == (nkz, 14)
    damped = "True" in data_comments[0]
    damp = float(data_comments[1].split(":")[1])
    spectra = sorted(os.path.join(ref_dir, "spectra", f) for f in os.listdir(ref_dir / "spectra")
                     if f.endswith(".dat"))
    # the input of the writers: the reference's printed numbers
    inp = tmp_path / "numbers.bin"
    with open(inp, "wb") as out:
        def vec(a):
            a = np.ascontiguousarray(a, dtype="<f8").ravel()
            out.write(struct.pack("<q", a.size))
            out.write(a.tobytes())
        vec(w.bins.k_edges)
        vec(w.bins.z_centers)
        out.write(struct.pack("<d", w.bins.dz))
        vec(np.asarray(w.fid, dtype=np.float64))
        out.write(struct.pack("<d", 0.0))
        out.write(struct.pack("<qd", int(damped), damp))
        vec(table[:, 5]); vec(table[:, 4]); vec(_matrix(ref[SUFFIXES[2]]))
        vec(table[:, 8:11].T); vec(table[:, 11:14].T)
        vec(_matrix(ref[SUFFIXES[1]])); vec(_matrix(ref[SUFFIXES[3]]))
        out.write(struct.pack("<q", len(spectra)))
        for p in spectra:
            b = p.encode()
            out.write(struct.pack("<q", len(b)))
            out.write(b)
    exe = str(tmp_path / "write_outputs")
    subprocess.run([gxx, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(HERE, "cpp", "write_outputs.cpp"), "-o", exe], check=True)
    base = str(tmp_path / "mine")
    r = subprocess.run([exe, str(inp), base], check=True, capture_output=True, text=True)
    pfid = np.array([float(x) for x in r.stdout.split()])
    # the fiducial power to the column's printing (7 significant digits)
    assert np.max(np.abs(pfid - table[:, 4]) / np.abs(table[:, 4])) <= 5e-7 * (1 + 1e-6)
    for s in SUFFIXES[1:]:
        assert open(base + "_it1" + s).read() == open(ref[s]).read(), s
    mine = open(base + "_it1" + SUFFIXES[0]).read().split("\n")
    j = next(k for k, ln in enumerate(mine) if ln.startswith("# Damping constant"))
    assert [ln for ln in mine if ln.startswith("# Damped")] + mine[j:j + 3] == data_comments
    counts = [int(c) for c in data_comments[3][1:].split()]
    assert counts[0] > 0 and sum(counts) == len(spectra)      # spectra out of range are counted too
    mbody = [ln for ln in mine if ln and not ln.startswith("#")]
    assert mbody[0] == body[0] and len(mbody) == len(body)
    for a, b in zip(mbody[1:], body[1:]):
        fa, fb = a.split(), b.split()
        assert [fa[k] for k in range(14) if k not in (6, 7)] == [fb[k] for k in range(14) if k not in (6, 7)]
        # Pest from the printed Pfid and ThetaP: their rounding, 5e-7 of each
        x, y = float(fa[6]), float(fb[6])
        assert abs(x - y) <= 1e-6 * (abs(float(fb[4])) + abs(float(fb[5]))), (a, b)
        # ErrorP from the printed inverse Fisher diagonal
        x, y = float(fa[7]), float(fb[7])
        assert (np.isnan(x) and np.isnan(y)) or abs(x - y) <= 1e-6 * abs(y), (a, b)
