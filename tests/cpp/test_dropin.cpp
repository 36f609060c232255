// lyspeq's own end-to-end test (tests/input/test.config, one binary spectrum,
// first iteration compared with tests/truth/test_it1_*), driven through the
// facade's constructors and calls with the reference's signatures:
//   OneQSOEstimate(const std::string &fname)
//   OneQSOEstimate::oneQSOiteration(ps_estimate, dbt_sum_vector, fisher_sum)
//   qio::QSOFile + Chunk(const qio::QSOFile &, int i1, int i2)
//   Chunk::oneQSOiteration(ps_estimate, dbt_sum_vector, fisher_sum)
// as OneDQuadraticPowerEstimate::iterate calls them (core/quadratic_estimate.cpp:
// 438-443), then invertTotalFisherMatrix.  Input: a binary file written by
// tests/test_cpp_facade.py (binning, table, options, the spectrum file's path,
// truth arrays).  Returns non-zero on a mismatch.
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
    std::string str() {
        std::string s(i64(), '\0');
        f.read(&s[0], s.size());
        return s;
    }
};

// tests/compareTestResults.py: |a - b| < 1e-8 + rel max(|a|, |b|)
bool close(double a, double b, double rel) { return std::fabs(a - b) < 1e-8 + rel * std::max(std::fabs(a), std::fabs(b)); }

int fails = 0;
void expect(bool ok, const std::string &what) {
    if (!ok) {
        std::printf("MISMATCH %s\n", what.c_str());
        ++fails;
    }
}

}  // namespace

int main(int argc, char **argv) {
    if (argc < 4) {
        std::fprintf(stderr, "usage: test_dropin <case.bin> <precision 0|1|2|3> <relative tolerance>\n");
        return 2;
    }
    Reader r(argv[1]);
    const int precision = std::atoi(argv[2]);
    const double tol = std::atof(argv[3]);
    Binning bins;
    bins.k_edges = r.vec();
    bins.z_centers = r.vec();
    bins.z_bin_width = r.f64();
    bins.triangular = r.i64() != 0;
    SQGrid grid;
    grid.nv = (int) r.i64();
    grid.v_length = r.f64();
    grid.nzp = (int) r.i64();
    SQTable t;
    t.r_fwhm = (int) r.i64();
    t.dv = r.f64();
    t.deriv = r.vec();
    t.signal = r.vec();
    Specifics sp;
    sp.max_forest_length = r.f64();
    sp.cont_logl_order = (int) r.i64();
    sp.cont_l_order = (int) r.i64();
    for (double &x : sp.fiducial) x = r.f64();
    const std::string dat = r.str();
    const std::vector<double> detailed = r.vec();   // nkz x 10: Pfid ThetaP Pest ErrorP dw bw tw d b t
    const std::vector<double> fisher_halved = r.vec();
    if (!r.f) {
        std::fprintf(stderr, "cannot read %s\n", argv[1]);
        return 2;
    }

    OneDQuadraticPowerEstimate est(bins, grid, {t}, sp);
    est.chunk_precision = (Precision) precision;
    std::vector<std::string> logs;
    est.log = [&](const std::string &m) { logs.push_back(m); };
    const int nkz = bins.nkz();

    // the reference's construction from a file name
    OneQSOEstimate q(dat);
    expect(!q.chunks.empty(), "OneQSOEstimate(fname) made no chunk");
    std::vector<std::unique_ptr<double[]>> dbt;
    for (int i = 0; i < 3; ++i) dbt.emplace_back(new double[nkz]());
    std::vector<double> fsum((size_t) nkz * nkz, 0.0), theta(nkz, 0.0);
    q.oneQSOiteration(theta.data(), dbt, fsum.data());
    expect(!q.chunks.empty(), "chunk dropped by oneQSOiteration");

    // d, b, t sums and the halved, symmetric Fisher matrix against the truth.
    // The mixed path holds d, b + t and F to the bar per element, b and t each
    // to the bar of the larger of the two (its smaller trace keeps the 22-bit
    // trace products' absolute error), so it is checked on d, b + t and each
    // of b, t against max(|b|, |t|).
    const bool strict = precision == LQG_PRECISION_FP64;
    for (int i = 0; i < nkz; ++i) {
        const double *tr = &detailed[(size_t) i * 10];
        expect(close(dbt[0][i], tr[7], tol), "d[" + std::to_string(i) + "]");
        if (strict) {
            expect(close(dbt[1][i], tr[8], tol), "b[" + std::to_string(i) + "]");
            expect(close(dbt[2][i], tr[9], tol), "t[" + std::to_string(i) + "]");
        } else {
            const double scale = std::max(std::fabs(tr[8]), std::fabs(tr[9]));
            expect(close(dbt[1][i] + dbt[2][i], tr[8] + tr[9], tol), "b + t[" + std::to_string(i) + "]");
            expect(std::fabs(dbt[1][i] - tr[8]) < 1e-8 + tol * scale, "b[" + std::to_string(i) + "]");
            expect(std::fabs(dbt[2][i] - tr[9]) < 1e-8 + tol * scale, "t[" + std::to_string(i) + "]");
        }
    }
    for (int i = 0; i < nkz; ++i)
        for (int j = 0; j < nkz; ++j) {
            const double fij = 0.5 * (i <= j ? fsum[(size_t) i * nkz + j] : fsum[(size_t) j * nkz + i]);
            expect(close(fij, fisher_halved[(size_t) i * nkz + j], tol),
                   "F[" + std::to_string(i) + "][" + std::to_string(j) + "]");
        }

    // the same chunk through qio::QSOFile and Chunk(const qio::QSOFile &, i1, i2)
    qio::QSOFile qf(dat, qio::Binary);
    qf.readParameters();
    qf.readData();
    qf.maskOutliers();
    qf.cutBoundary(bins.z_lower(), bins.z_upper());
    Chunk ch(qf, 0, qf.size());
    std::vector<std::unique_ptr<double[]>> dbt2;
    for (int i = 0; i < 3; ++i) dbt2.emplace_back(new double[nkz]());
    std::vector<double> fsum2((size_t) nkz * nkz, 0.0);
    ch.oneQSOiteration(theta.data(), dbt2, fsum2.data());
    for (int i = 0; i < nkz; ++i)
        for (int k = 0; k < 3; ++k)
            expect(std::fabs(dbt2[k][i] - dbt[k][i]) <= 1e-12 * std::fabs(dbt[k][i]) + 1e-300, "Chunk vs OneQSOEstimate dbt");
    for (size_t e = 0; e < fsum.size(); ++e)
        expect(std::fabs(fsum2[e] - fsum[e]) <= 1e-12 * std::fabs(fsum[e]) + 1e-300, "Chunk vs OneQSOEstimate F");

    // invertTotalFisherMatrix + computePowerSpectrumEstimates on these sums
    for (int k = 0; k < 3; ++k) std::copy(dbt[k].get(), dbt[k].get() + nkz, est.dbt_estimate_sum_before_fisher_vector[k].get());
    std::copy(fsum.begin(), fsum.end(), est.fisher_matrix_sum.get());
    est.invertTotalFisherMatrix();
    for (int i = 0; i < nkz; ++i) {
        expect(close(est.current_power_estimate_vector[i], detailed[(size_t) i * 10 + 1], tol),
               "ThetaP[" + std::to_string(i) + "] " + std::to_string(est.current_power_estimate_vector[i]) + " vs " +
                   std::to_string(detailed[(size_t) i * 10 + 1]));
        expect(close(std::sqrt(est.inverse_fisher_matrix_sum[(size_t) i * (nkz + 1)]), detailed[(size_t) i * 10 + 3], tol),
               "ErrorP[" + std::to_string(i) + "]");
        const double *w = &detailed[(size_t) i * 10 + 4];
        const double dw = est.dbt_estimate_fisher_weighted_vector[0][i], bw = est.dbt_estimate_fisher_weighted_vector[1][i],
                     tw = est.dbt_estimate_fisher_weighted_vector[2][i];
        expect(close(dw, w[0], tol), "Fisher-weighted d[" + std::to_string(i) + "]");
        if (strict) {
            expect(close(bw, w[1], tol), "Fisher-weighted b[" + std::to_string(i) + "]");
            expect(close(tw, w[2], tol), "Fisher-weighted t[" + std::to_string(i) + "]");
        } else {
            expect(close(bw + tw, w[1] + w[2], tol), "Fisher-weighted b + t[" + std::to_string(i) + "]");
        }
    }
    for (const auto &m : logs) std::printf("log: %s\n", m.c_str());
    std::printf("%s: %d mismatches\n", fails ? "FAILED" : "ok", fails);
    return fails ? 1 : 0;
}
