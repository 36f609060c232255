"""C++ facade (include/lyspeq_api.hpp) driven by a C++ test program
(tests/cpp/test_facade.cpp) the way lyspeq's own tests drive its classes: the
tiny workload's spectra go through OneQSOEstimate chunking and one FP64
Newton-Raphson iteration, compared with the CPU restatement of lyspeq's path
(global Fisher matrix, d/b/t sums, theta and every chunk's own results); then
the FastBootstrap after that iteration and a 4-iteration loop with smoothing,
compared with lyspeq's own results (golden fixtures tiny_boot, tiny_iter)."""
import os
import shutil
import struct
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _write(path, w, s, chunks, results, g):
    from oracle import qmle_port as P
    out = open(path, "wb")
    i64 = lambda v: out.write(struct.pack("<q", int(v)))
    f64 = lambda v: out.write(struct.pack("<d", float(v)))

    def vec(a):
        a = np.ascontiguousarray(a, dtype="<f8").ravel()
        i64(a.size)
        out.write(a.tobytes())

    vec(w.bins.k_edges); vec(w.bins.z_centers); f64(w.bins.dz); i64(1 if w.bins.triangular else 0)
    i64(w.nv); f64(w.lenv); i64(w.nzp)
    i64(len(w.tables))
    for t in w.tables:
        i64(t.r_fwhm); f64(t.dv); vec(t.deriv); vec(t.signal)
    f64(s.max_forest_length); i64(s.cont_logl_order); i64(s.cont_l_order)
    i64(len(w.spectra))
    for sp in w.spectra:
        i64(sp.r_fwhm); vec(sp.wave); vec(sp.delta); vec(1.0 / np.asarray(sp.sigma, dtype=np.float64) ** 2)
    i64(len(chunks))
    fsum = g["fsum"]
    vec(fsum); vec(g["dbt"]); vec(g["theta"])
    for d, b, t, f in results:
        vec(np.concatenate([d, b, t])); vec(f)
    out.close()


def test_cpp_program_compiles_against_the_header():
    """Host-only: the facade and the test program compile and link."""
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    from lyspeq_gb300 import build
    lib = build.build()
    exe = os.path.join(HERE, "cpp", "test_facade")
    subprocess.run([gxx, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(HERE, "cpp", "test_facade.cpp"), "-L", os.path.dirname(lib), "-llqg",
                    "-Wl,-rpath," + os.path.dirname(lib), "-o", exe], check=True)
    assert os.path.exists(exe)


@pytest.mark.gpu
def test_cpp_facade_one_iteration_matches_the_oracle(tmp_path):
    from lyspeq_gb300 import build, synth
    from oracle import qmle_port as P

    gxx = shutil.which("g++")
    lib = build.build()
    exe = os.path.join(HERE, "cpp", "test_facade")
    subprocess.run([gxx, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(HERE, "cpp", "test_facade.cpp"), "-L", os.path.dirname(lib), "-llqg",
                    "-Wl,-rpath," + os.path.dirname(lib), "-o", exe], check=True)
    w = synth.make_workload("tiny")
    s = P.Settings(max_forest_length=w.max_forest_length, cont_logl_order=1, cont_l_order=-1)
    chunks = P.chunks_from_spectra(w.spectra, w.bins, w.table_index(), s)
    tvs = [P.table_view(t, w.bins, w.nv, w.lenv, w.nzp) for t in w.tables]
    results, acc = [], []
    for ch in chunks:
        d, b, t, f = P.chunk_iteration(ch, w.bins, tvs[ch.res_index], np.zeros(w.bins.nkz), s)
        results.append((d, b, t, f))
        acc.append((ch.fisher_index_start, d, b, t, f))
    fsum, dbt = P.accumulate(w.bins.nkz, acc)
    nr = P.newton_raphson_step(fsum, dbt)
    path = str(tmp_path / "case.bin")
    _write(path, w, s, chunks, results, dict(fsum=fsum, dbt=dbt, theta=nr["theta"]))
    # lyspeq's own NR loop (4 iterations) and FastBootstrap (200) on these spectra
    import sys
    import golden_cases as G
    it, bt = G.load("tiny_iter").nr, G.load("tiny_boot").boot
    loop = str(tmp_path / "loop.bin")
    with open(loop, "wb") as f:
        def blob(b):
            f.write(struct.pack("<q", len(b)))
            f.write(b)

        def vec(a):
            a = np.ascontiguousarray(a, dtype="<f8").ravel()
            f.write(struct.pack("<q", a.size))
            f.write(a.tobytes())
        blob(f"cd {ROOT} && {sys.executable} -m lyspeq_gb300.smoothing".encode())
        blob(str(tmp_path).encode())
        f.write(struct.pack("<q", it["n"]))
        vec(it["theta"]); vec(it["fits"])
        f.write(struct.pack("<q", bt["real"].shape[0]))
        vec(bt["mean"]); vec(bt["cov"])
    r = subprocess.run([exe, path, "1e-9", loop], capture_output=True, text=True)
    print(r.stdout, r.stderr)
    assert r.returncode == 0, r.stdout + r.stderr


@pytest.mark.parametrize("workload", ["tiny", "small"])
def test_cpp_chunking_matches_the_oracle(tmp_path, workload):
    """Host-only: the facade's OneQSOEstimate::decideIndices cuts every cleaned
    spectrum of the workload where the restatement's decide_indices does
    (itself pinned to the compiled reference's chunks in tests/test_oracle.py),
    for DynamicChunkNumber 1 to 3."""
    from lyspeq_gb300 import build, synth
    from oracle import qmle_port as P
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    lib = build.build()
    exe = str(tmp_path / "decide_indices")
    subprocess.run([gxx, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(HERE, "cpp", "decide_indices.cpp"), "-L", os.path.dirname(lib), "-llqg",
                    "-Wl,-rpath," + os.path.dirname(lib), "-o", exe], check=True)
    w = synth.make_workload(workload)
    waves = []
    for s in w.spectra:
        try:
            waves.append(P.preprocess_spectrum(s, w.bins)[0])
        except ValueError:
            continue
    cases, want = [], []
    for nch in (1, 2, 3):
        st = P.Settings(max_forest_length=w.max_forest_length, number_of_chunks=nch)
        for wave in waves:
            cases.append((w.max_forest_length, nch, wave))
            want.append(P.decide_indices(wave, st))
    path = tmp_path / "waves.bin"
    with open(path, "wb") as out:
        out.write(struct.pack("<q", len(cases)))
        for mfl, nch, wave in cases:
            out.write(struct.pack("<dqq", mfl, nch, len(wave)))
            out.write(np.ascontiguousarray(wave, dtype="<f8").tobytes())
    r = subprocess.run([exe, str(path)], capture_output=True, text=True, check=True)
    got = [[int(x) for x in ln.split()] for ln in r.stdout.strip().split("\n")]
    assert got == want
    assert any(len(idx) > 2 for idx in want)      # some spectra were split


def _compile(name):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    from lyspeq_gb300 import build
    lib = build.build()
    exe = os.path.join(HERE, "cpp", name)
    subprocess.run([gxx, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(HERE, "cpp", name + ".cpp"), "-L", os.path.dirname(lib), "-llqg",
                    "-Wl,-rpath," + os.path.dirname(lib), "-o", exe], check=True)
    return exe


def test_dropin_program_compiles_against_the_header():
    """Host-only: the reference-signature drop-in program compiles and links."""
    assert os.path.exists(_compile("test_dropin"))


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [(0, 1e-5), (1, 1e-5)])
def test_reference_signatures_reproduce_lyspeqs_own_test(engine_lib, tmp_path, precision, tol):
    """lyspeq's end-to-end test (its spectrum file and test.config, truth
    test_it1_*: fixture lyspeq_test_it1) through OneQSOEstimate(fname),
    Chunk(QSOFile, i1, i2) and their oneQSOiteration with the reference's
    signatures, at the reference's own comparison tolerance
    (tests/compareTestResults.py: 1e-8 absolute + 1e-5 relative)."""
    from lyspeq_gb300 import synth
    exe = _compile("test_dropin")
    z = np.load(os.path.join(HERE, "golden", "lyspeq_test_it1.npz"))
    b = z["bins"]
    bins = synth.Bins(b[0], int(b[1]), b[2], int(b[3]), b[4], b[5], b[6], int(b[7]))
    nv, lenv, nzp, mfl, c0, c1 = z["grid"]
    fid = tuple(float(x) for x in z["fid"])
    r, dv = z["tables"][0]
    table = synth.build_table(bins, int(r), float(dv), int(nv), float(lenv), int(nzp), fid=fid)
    dat = tmp_path / "spectrum.dat"
    dat.write_bytes(z["dat"].tobytes())
    path = tmp_path / "case.bin"
    with open(path, "wb") as out:
        i64 = lambda v: out.write(struct.pack("<q", int(v)))
        f64 = lambda v: out.write(struct.pack("<d", float(v)))

        def vec(a):
            a = np.ascontiguousarray(a, dtype="<f8").ravel()
            i64(a.size)
            out.write(a.tobytes())

        vec(bins.k_edges); vec(bins.z_centers); f64(bins.dz); i64(1)
        i64(nv); f64(lenv); i64(nzp)
        i64(int(r)); f64(dv); vec(table.deriv); vec(table.signal)
        f64(mfl); i64(c0); i64(c1)
        for x in fid:
            f64(x)
        s = str(dat).encode()
        i64(len(s)); out.write(s)
        vec(z["detailed"]); vec(z["fisher_halved"])
    res = subprocess.run([exe, str(path), str(precision), str(tol)], capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stdout[-4000:] + res.stderr[-2000:]
