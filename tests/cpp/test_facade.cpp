// C++ parity test of the facade (include/lyspeq_api.hpp), in the manner of
// lyspeq's own test programs (tests/testOneQSOEstimate.cpp,
// tests/testSQCMatrices.cpp): build the estimator from tables and spectra,
// run one Newton-Raphson iteration, compare with expected arrays, return
// non-zero on a mismatch.  Input: one binary file written by
// tests/test_cpp_facade.py (spectra, tables, binning, expected results of the
// CPU restatement of lyspeq's path) and optionally a second one with lyspeq's
// own bootstrap and multi-iteration results on the same spectra.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <fstream>
#include <string>
#include <vector>

#include "lyspeq_api.hpp"

using namespace lyspeq_gb300;

namespace {

struct Reader {
    std::ifstream f;
    explicit Reader(const char *path) : f(path, std::ios::binary) {}
    int64_t i64() { int64_t v; f.read(reinterpret_cast<char *>(&v), 8); return v; }
    double f64() { double v; f.read(reinterpret_cast<char *>(&v), 8); return v; }
    std::vector<double> vec() {
        std::vector<double> v(i64());
        f.read(reinterpret_cast<char *>(v.data()), v.size() * 8);
        return v;
    }
    bool ok() const { return (bool) f; }
};

double rel_err(const double *x, const double *ref, size_t n) {
    double scale = 0, err = 0;
    for (size_t i = 0; i < n; ++i) scale = std::max(scale, std::fabs(ref[i]));
    for (size_t i = 0; i < n; ++i) err = std::max(err, std::fabs(x[i] - ref[i]));
    return scale > 0 ? err / scale : err;
}

// Fisher elements normalised by sqrt(F_ii F_jj)
double fisher_err(const double *f, const double *ref, int n) {
    double e = 0;
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
            double d = std::sqrt(std::fabs(ref[i * n + i] * ref[j * n + j]));
            if (d == 0) d = 1;
            e = std::max(e, std::fabs(f[i * n + j] - ref[i * n + j]) / d);
        }
    return e;
}

}  // namespace

int main(int argc, char **argv) {
    if (argc < 3) {
        std::fprintf(stderr, "usage: test_facade <case.bin> <tolerance> [<loop.bin>]\n");
        return 2;
    }
    const double tol = std::stod(argv[2]);
    Reader r(argv[1]);
    Binning bins;
    bins.k_edges = r.vec();
    bins.z_centers = r.vec();
    bins.z_bin_width = r.f64();
    bins.triangular = r.i64() != 0;
    SQGrid grid;
    grid.nv = (int) r.i64();
    grid.v_length = r.f64();
    grid.nzp = (int) r.i64();
    std::vector<SQTable> tables(r.i64());
    for (auto &t : tables) {
        t.r_fwhm = (int) r.i64();
        t.dv = r.f64();
        t.deriv = r.vec();
        t.signal = r.vec();
    }
    Specifics sp;
    sp.max_forest_length = r.f64();
    sp.cont_logl_order = (int) r.i64();
    sp.cont_l_order = (int) r.i64();
    std::vector<QSOSpectrum> spectra(r.i64());
    for (auto &q : spectra) {
        q.r_fwhm = (int) r.i64();
        q.wave = r.vec();
        q.delta = r.vec();
        q.ivar = r.vec();
    }
    const int64_t nchunks_expected = r.i64();
    const std::vector<double> fisher_ref = r.vec(), dbt_ref = r.vec(), theta_ref = r.vec();
    std::vector<std::vector<double>> chunk_d(nchunks_expected), chunk_f(nchunks_expected);
    for (int64_t i = 0; i < nchunks_expected; ++i) {
        chunk_d[i] = r.vec();
        chunk_f[i] = r.vec();
    }
    if (!r.ok()) {
        std::fprintf(stderr, "could not read %s\n", argv[1]);
        return 2;
    }

    OneDQuadraticPowerEstimate qe(bins, grid, tables, sp);
    for (const auto &q : spectra) qe.addQSO(q);
    int nch = 0;
    for (const auto &q : qe.local_queue) nch += (int) q->chunks.size();
    std::printf("spectra %zu, chunks %d (expected %lld)\n", spectra.size(), nch, (long long) nchunks_expected);
    if (nch != nchunks_expected) return 1;

    qe.iterate(1, Precision::FP64);
    qe.fetchResults();
    const int nkz = bins.nkz();
    const double ef = fisher_err(qe.fisher_matrix_sum.get(), fisher_ref.data(), nkz);
    double edbt = 0;
    for (int i = 0; i < 3; ++i)
        edbt = std::max(edbt, rel_err(qe.dbt_estimate_sum_before_fisher_vector[i].get(), dbt_ref.data() + i * nkz, nkz));
    const double eth = rel_err(qe.current_power_estimate_vector.get(), theta_ref.data(), nkz);
    double ech = 0;
    int k = 0;
    for (const auto &q : qe.local_queue)
        for (const auto &ch : q->chunks) {
            const int nq = ch->N_Q_MATRICES;
            for (int i = 0; i < 3; ++i)
                ech = std::max(ech, rel_err(ch->dbt_estimate_before_fisher_vector[i].get(), chunk_d[k].data() + i * nq, nq));
            ech = std::max(ech, fisher_err(ch->fisher_matrix.get(), chunk_f[k].data(), nq));
            ++k;
        }
    std::printf("max rel err: global fisher %.2e, dbt %.2e, theta %.2e, per chunk %.2e (tolerance %.1e)\n", ef,
                edbt, eth, ech, tol);
    bool ok = ef < tol && edbt < tol && eth < tol && ech < tol;
    if (argc > 3) {
        // lyspeq's own NR loop and FastBootstrap on these spectra (expected values
        // from the reference): iterate(N) with smoothing, bootstrap(nboots) after
        // the single iteration above
        Reader r2(argv[3]);
        auto str = [&r2]() {
            std::string t(r2.i64(), ' ');
            r2.f.read(&t[0], t.size());
            return t;
        };
        const std::string cmd = str(), tmp = str();
        const int niter = (int) r2.i64();
        const std::vector<double> theta_it = r2.vec(), fits_it = r2.vec();
        const int nboots = (int) r2.i64();
        const std::vector<double> boot_mean = r2.vec(), boot_cov = r2.vec();
        if (!r2.ok()) {
            std::fprintf(stderr, "could not read %s\n", argv[3]);
            return 2;
        }
        qe.bootstrap(nboots, 0);
        const double ebm = rel_err(qe.bootstrap_mean.data(), boot_mean.data(), nkz);
        const double ebc = rel_err(qe.bootstrap_covariance.data(), boot_cov.data(), (size_t) nkz * nkz);
        Specifics sp2 = sp;
        sp2.smooth_logk_logp = false;
        sp2.smoothing_command = cmd;
        sp2.tmp_folder = tmp;
        OneDQuadraticPowerEstimate qe2(bins, grid, tables, sp2);
        for (const auto &q : spectra) qe2.addQSO(q);
        const int its = qe2.iterate(niter, Precision::FP64);
        const double eit = rel_err(qe2.current_power_estimate_vector.get(), theta_it.data(), nkz);
        const double efit = rel_err(qe2.powerspectra_fits.get(), fits_it.data(), nkz);
        std::printf("bootstrap: mean %.2e, covariance %.2e; NR loop (%d iterations): theta %.2e, fits %.2e\n", ebm,
                    ebc, its, eit, efit);
        ok = ok && ebm < 1e-10 && ebc < 1e-9 && eit < 1e-8 && efit < 1e-8;
    }
    return ok ? 0 : 1;
}
