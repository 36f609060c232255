// lyspeq_api.hpp - C++ facade of the GB300 engine with lyspeq's class names.
//
// lyspeq's per-chunk path is a C++ class API (no FFI).  This header keeps its
// shape on top of the C ABI of lqg.h, so that a lyspeq-style driver reads the
// same with the engine underneath:
//
//   lyspeq                                            here
//   qio::QSOFile (binary .dat files)                  qio::QSOFile (same reading steps);
//     (io/qso_file.cpp:37-230, 334-369)                 QSOSpectrum for arrays in memory
//   OneQSOEstimate(const std::string &fname)          same signature, and addQSO(spectrum)
//     (core/one_qso_estimate.cpp:52-121)
//   Chunk(const qio::QSOFile&, int i1, int i2)        same signature
//     (core/chunk_estimate.cpp:141-257)
//   Chunk::oneQSOiteration(ps, dbt_sum, fisher_sum)   same signature: the first call for a theta
//   OneQSOEstimate::oneQSOiteration(same)               runs one batched iteration of every chunk
//     (core/chunk_estimate.cpp:837-914,                 on the GPU; each call then adds its own
//      core/one_qso_estimate.cpp:176-197)               chunk's results to the caller's sums
//   Chunk::dbt_estimate_before_fisher_vector,         same members, filled after iterate()
//     Chunk::fisher_matrix                              (fetchResults())
//   OneDQuadraticPowerEstimate::iterate()             same name; one batched NR iteration per
//     (core/quadratic_estimate.cpp:398-546)             iteration on the GPU
//   ::invertTotalFisherMatrix / ::computePowerSpectrumEstimates (:261-318)
//   fisher_matrix_sum, inverse_fisher_matrix_sum,     same members
//     solver_invfisher_matrix,
//     dbt_estimate_sum_before_fisher_vector,
//     dbt_estimate_fisher_weighted_vector,
//     current_power_estimate_vector, powerspectra_fits
//
// Errors follow the reference: a spectrum or chunk the reference rejects
// with an exception is skipped (logged through the optional log callback),
// and a failure of the engine throws std::runtime_error.  Like the
// reference's process-wide tables and settings, the constructors with the
// reference's signatures use the process's current estimator: the last
// OneDQuadraticPowerEstimate constructed (not thread safe, as the reference).
//
// Header-only; link with -llqg (lyspeq_gb300/liblqg.so).
#ifndef LYSPEQ_API_HPP
#define LYSPEQ_API_HPP

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cstdint>
#include <functional>
#include <memory>
#include <numeric>
#include <stdexcept>
#include <string>
#include <vector>

#include "lqg.h"

namespace lyspeq_gb300 {

constexpr double SPEED_OF_LIGHT = 299792.458;   // core/global_numbers.hpp
constexpr double LYA_REST = 1215.67;
constexpr int MIN_PIXELS_IN_FILE = 100;         // core/one_qso_estimate.cpp:14

enum class Precision {
    FP64 = LQG_PRECISION_FP64,
    Mixed = LQG_PRECISION_MIXED,
    MixedDirect = LQG_PRECISION_MIXED_DIRECT,
    MixedAuto = LQG_PRECISION_MIXED_AUTO   // the autotuned plan (autotune(), loadTuning())
};

// bins:: (core/global_numbers.cpp:209-251)
struct Binning {
    std::vector<double> k_edges;    // NUMBER_OF_K_BANDS + 1
    std::vector<double> z_centers;  // NUMBER_OF_Z_BINS
    double z_bin_width = 0.2;
    bool triangular = true;         // RedshiftBinningMethod 1
    int nk() const { return (int) k_edges.size() - 1; }
    int nz() const { return (int) z_centers.size(); }
    int nkz() const { return nk() * nz(); }
    double z_lower() const { return z_centers.front() - z_bin_width / 2; }
    double z_upper() const { return z_centers.back() + z_bin_width / 2; }
    // bins::findRedshiftBin (core/global_numbers.cpp:344-355): -1 below the
    // first bin, NUMBER_OF_Z_BINS above the last
    int findRedshiftBin(double z) const {
        if (z < z_lower()) return -1;
        return std::min((int) ((z - z_lower()) / z_bin_width), nz());
    }
};

// One (R, dv) pair of SQ lookup tables (SQLookupTable, core/sq_table.cpp):
// deriv[k][v] (nk x nv) and signal[v][z] (nv x nzp).
struct SQTable {
    int r_fwhm = 0;
    double dv = 0;
    std::vector<double> deriv, signal;
};

struct SQGrid {
    int nv = 0;           // NumberVPoints
    double v_length = 0;  // VelocityLength
    int nzp = 0;          // NumberZPoints
};

// The specifics:: values of the path (core/global_numbers.cpp:93-173).
struct Specifics {
    double max_forest_length = 35000;   // MaximumForestLength
    int number_of_chunks = 1;           // DynamicChunkNumber
    double max_mean_pixel_size = 150;   // MaximumMeanPixelSize (MAX_PIXEL_LENGTH_V)
    int cont_logl_order = 1;            // ContinuumLogLambdaMargOrder
    int cont_l_order = -1;              // ContinuumLambdaMargOrder
    bool turn_off_sfid = false;         // TurnOffBaseline
    bool precomputed_fisher = false;    // PrecomputedFisher given (no Fisher matrices computed)
    std::string precomputed_fisher_file;  // PrecomputedFisher: its file, used in place of the sum
    double chisq_convergence = 0.01;    // ChiSqConvergence (CHISQ_CONVERGENCE_EPS)
    bool smooth_logk_logp = true;       // SmoothLnkLnP
    // the six PD13 fiducial parameters (FiducialAmplitude, ...Slope, ...Curvature,
    // ...RedshiftPower, ...RedshiftCurvature, ...LorentzianLambda)
    double fiducial[6] = {6.621420e-02, -2.685349e+00, -2.232763e-01, 3.591244e+00, -1.768045e-01, 3.598261e+02};
    // the smoothing command between iterations (lyspeq runs its smbivspline.py)
    std::string smoothing_command = "python3 -m lyspeq_gb300.smoothing";
    std::string tmp_folder = ".";       // TemporaryFolder
    bool use_reso_matrix = false;       // UseResoMatrix
    int oversampling = -1;              // OversampleRmat
    double resomat_deconvolution_m = 0; // ResoMatDeconvolutionM
    int smooth_noise_weights = -1;      // SmoothNoiseWeights
    bool smooth_resolution_matrix = false;  // SmoothResolutionMatrix > 0 (needs SmoothNoiseWeights >= 0)
    bool redshift_growth_on = false;    // RedshiftGrowthOn > 0 (exponent: fiducial[3])
    double min_snr_cut = 0;             // MinimumSnrCut
    // flux -> delta_F of the input (conv::readConversion, core/fiducial_cosmology.cpp:33-83)
    bool input_is_delta_flux = true;    // InputIsDeltaFlux > 0
    bool use_chunks_mean_flux = false;  // UseChunksMeanFlux > 0
    std::string mean_flux_file;         // MeanFluxFile (binary: int32 n, n doubles z, n doubles F-bar)
    // OutputDir / OutputFileBase: with a base name set, every iteration writes
    // <dir>/<base>_it<N>_{quadratic_power_estimate_detailed, fisher_matrix,
    // inversefisher_matrix, solver_invfishermatrix}.txt as the reference does
    std::string output_dir = ".";
    std::string output_file_base;
    double max_forest_length_v() const { return max_forest_length / std::max(1, number_of_chunks); }
};

// The PD13 fit with a Lorentzian factor (Palanque_Delabrouille_etal_2013_fit,
// core/fiducial_cosmology.cpp:273-282); p = A, n, alpha, B, beta, lambda,
// k0 = 0.009 s/km, z0 = 3.
inline double fiducialPowerPD13(double k, double z, const double p[6]) {
    const double q0 = k / 0.009 + 1e-15, x0 = (1. + z) / (1. + 3.0);
    return (p[0] * 3.14159265358979323846 / 0.009) *
           std::pow(q0, 2. + p[1] + p[2] * std::log(q0) + p[4] * std::log(x0)) * std::pow(x0, p[3]) /
           (1. + p[5] * k * k);
}

// A spectrum as qio::QSOFile holds it after reading: observed wavelength in
// Angstrom, flux contrast and inverse variance (0 = masked), resolution R.
struct QSOSpectrum {
    std::vector<double> wave, delta, ivar;
    int r_fwhm = 0;
    // resolution matrix (UseResoMatrix), DiaMatrix layout resomat[ndiags][n]:
    // diagonal d holds offset ndiags / 2 - d, its entry of column c at [d][c]
    std::vector<double> resomat;
    int ndiags = 0;
};

namespace qio {

enum ifileformat { Binary, Picca };

// A spectrum file as lyspeq's qio::QSOFile reads it.  Binary files only
// (qio::BQFile, io/qso_file.cpp:334-369): an 88-byte header (int size, double
// z, dec, ra, int R_fwhm, double S/N, pixel width in km/s, lower and upper
// observed and rest wavelengths; C struct layout) and then size doubles each
// of lambda (Angstrom), delta and sigma; ivar = 1 / sigma^2, 0 below 1e-15.
// picca FITS files are not read by this build.
class QSOFile {
public:
    std::string fname;
    double z_qso = 0, snr = 0, dv_kms = -1, dlambda = -1, ra = 0, dec = 0, R_kms = 0;
    int R_fwhm = 0;
    long id = 0;

    QSOFile(const std::string &fname_qso, ifileformat p_or_b = Binary) : fname(fname_qso) {
        if (p_or_b != Binary) throw std::runtime_error("QSOFile: picca FITS input is not supported");
    }
    // A slice [i1, i2) of a read file with its masked ends removed
    // (QSOFile::QSOFile(qmaster, i1, i2), io/qso_file.cpp:61-89)
    QSOFile(const QSOFile &q, int i1, int i2)
        : fname(q.fname), z_qso(q.z_qso), snr(q.snr), ra(q.ra), dec(q.dec), R_kms(q.R_kms), R_fwhm(q.R_fwhm),
          id(q.id) {
        if (i1 < 0 || i2 > q.size() || i2 <= i1) throw std::out_of_range("QSOFile: slice out of range");
        w_.assign(q.wave() + i1, q.wave() + i2);
        d_.assign(q.delta() + i1, q.delta() + i2);
        iv_.assign(q.ivar() + i1, q.ivar() + i2);
        first_ = 0;
        n_ = i2 - i1;
        cutMaskedBoundary();
        recalc();
    }

    // QSOFile::readParameters + BQFile::readParameters (io/qso_file.cpp:91-105, 334-351)
    void readParameters() {
        std::FILE *f = std::fopen(fname.c_str(), "rb");
        if (!f) throw std::runtime_error("QSOFile: cannot open " + fname);
        unsigned char h[88];
        const bool ok = std::fread(h, 1, 88, f) == 88;
        std::fclose(f);
        if (!ok) throw std::runtime_error("fread error in header BQFile!");
        auto i32 = [&](int off) { int v; std::memcpy(&v, h + off, 4); return v; };
        auto f64 = [&](int off) { double v; std::memcpy(&v, h + off, 8); return v; };
        n_file_ = i32(0);
        z_qso = f64(8); dec = f64(16); ra = f64(24);
        R_fwhm = i32(32);
        snr = f64(40); dv_kms = f64(48);
        R_kms = SPEED_OF_LIGHT / R_fwhm / ONE_SIGMA_2_FWHM;
    }

    // QSOFile::readData + BQFile::readData (io/qso_file.cpp:107-129, 353-369)
    void readData() {
        if (n_file_ <= 0) throw std::runtime_error("File is non-positive!");
        std::FILE *f = std::fopen(fname.c_str(), "rb");
        if (!f) throw std::runtime_error("QSOFile: cannot open " + fname);
        w_.resize(n_file_); d_.resize(n_file_); iv_.resize(n_file_);
        bool ok = std::fseek(f, 88, SEEK_SET) == 0;
        ok = ok && std::fread(w_.data(), 8, n_file_, f) == (size_t) n_file_;
        ok = ok && std::fread(d_.data(), 8, n_file_, f) == (size_t) n_file_;
        ok = ok && std::fread(iv_.data(), 8, n_file_, f) == (size_t) n_file_;
        std::fclose(f);
        if (!ok) throw std::runtime_error("fread error in data BQFile!");
        for (auto &x : iv_) {
            x = 1.0 / (x * x);
            if (x < 1e-15) x = 0;
        }
        first_ = 0;
        n_ = n_file_;
        if (dlambda < 0 || dv_kms < 0) recalc();
    }

    void closeFile() {}

    int size() const { return n_; }
    int realSize() const {
        return (int) std::count_if(iv_.begin() + first_, iv_.begin() + first_ + n_, [](double x) { return x != 0; });
    }
    const double *wave() const { return w_.data() + first_; }
    const double *delta() const { return d_.data() + first_; }
    const double *ivar() const { return iv_.data() + first_; }
    double *wave() { return w_.data() + first_; }
    double *delta() { return d_.data() + first_; }
    double *ivar() { return iv_.data() + first_; }

    // QSOFile::maskOutliers (io/qso_file.cpp:189-230); returns the number masked
    int maskOutliers(double factor = 5.0) {
        std::vector<double> tmp;
        for (int i = 0; i < n_; ++i)
            if (ivar()[i] != 0) tmp.push_back(delta()[i]);
        if (tmp.empty()) return 0;
        const double med = median(tmp);
        for (auto &x : tmp) x = std::fabs(x - med);
        double mad = 1.4826 * (1.0 + 1.0 / std::sqrt((double) tmp.size())) * median(tmp);
        mad = std::max(1.0, mad);
        int j = 0;
        for (int i = 0; i < n_; ++i) {
            double &iv = ivar()[i], &f = delta()[i];
            if (iv == 0) continue;
            const double s = factor * std::max(1.0 / std::sqrt(iv), mad);
            const double fup = std::exp(1.663e-03 * std::pow(wave()[i] / LYA_REST, 4.107));
            if (f < (-1.0 - s) || f > (fup + s)) {
                f = 0;
                iv = 0;
                ++j;
            }
        }
        return j;
    }

    // QSOFile::cutBoundary (io/qso_file.cpp:159-187)
    void cutBoundary(double z_lower_edge, double z_upper_edge) {
        const double l1 = LYA_REST * (1 + z_lower_edge), l2 = LYA_REST * (1 + z_upper_edge);
        const int wi1 = (int) (std::lower_bound(wave(), wave() + n_, l1) - wave());
        const int wi2 = (int) (std::upper_bound(wave(), wave() + n_, l2) - wave());
        if (wi1 == n_ || wi2 == 0) throw std::runtime_error("Empty spectrum when redshift boundary is applied!");
        first_ += wi1;
        n_ = wi2 - wi1;
        cutMaskedBoundary();
    }

    static double median(std::vector<double> v) {
        std::sort(v.begin(), v.end());
        const size_t n = v.size();
        return n % 2 == 0 ? (v[n / 2 - 1] + v[n / 2]) / 2 : v[n / 2];
    }

    static constexpr double ONE_SIGMA_2_FWHM = 2.35482004503;

private:
    std::vector<double> w_, d_, iv_;
    int first_ = 0, n_ = 0, n_file_ = 0;

    // QSOFile::_cutMaskedBoundary (io/qso_file.cpp:139-157)
    void cutMaskedBoundary() {
        int a = 0, b = n_;
        while (a < n_ && ivar()[a] == 0) ++a;
        while (b > 0 && ivar()[b - 1] == 0) --b;
        if (b - a <= 0) throw std::runtime_error("Empty spectrum when masked pixels at boundary are removed!");
        first_ += a;
        n_ = b - a;
    }

    // QSOFile::recalcDvDLam (io/qso_file.cpp:325-329): median pixel widths
    void recalc() {
        if (n_ < 2) return;
        std::vector<double> dl(n_ - 1), dv(n_ - 1);
        for (int i = 0; i + 1 < n_; ++i) {
            dl[i] = wave()[i + 1] - wave()[i];
            dv[i] = SPEED_OF_LIGHT * std::log(wave()[i + 1] / wave()[i]);
        }
        dlambda = median(dl);
        dv_kms = median(dv);
    }
};

}  // namespace qio

// Flux to flux contrast, lyspeq's conv:: (core/fiducial_cosmology.cpp:18-169),
// applied to a whole spectrum after reading and before its outliers are
// masked (core/one_qso_estimate.cpp:62-65).
namespace conv {

enum class Conversion { None, ChunkMean, MeanFluxFile };

// conv::readConversion's resolution of the three keys: delta input wins over
// both conversions, the spectrum's own mean over a mean-flux file; with none
// of them set the input is taken as delta.
inline Conversion conversion(const Specifics &sp) {
    if (sp.input_is_delta_flux) return Conversion::None;
    if (sp.use_chunks_mean_flux) return Conversion::ChunkMean;
    if (!sp.mean_flux_file.empty()) return Conversion::MeanFluxFile;
    return Conversion::None;
}

// Mean flux F-bar(z) of a MeanFluxFile (conv::setMeanFlux, :131-165): the
// natural cubic spline through its points (GSL_CUBIC_INTERPOLATION), continued
// past either end along its end slope (Interpolation::evaluate,
// mathtools/interpolation.cpp:42-62).
class MeanFlux {
public:
    MeanFlux(std::vector<double> z, std::vector<double> f) : x_(std::move(z)), y_(std::move(f)) { init(); }
    explicit MeanFlux(const std::string &fname) {
        std::FILE *fp = std::fopen(fname.c_str(), "rb");
        if (!fp) throw std::runtime_error("MeanFluxFile: cannot open " + fname);
        int32_t n = 0;
        bool ok = std::fread(&n, 4, 1, fp) == 1 && n > 0;
        if (ok) {
            x_.resize(n);
            y_.resize(n);
            ok = std::fread(x_.data(), 8, n, fp) == (size_t) n && std::fread(y_.data(), 8, n, fp) == (size_t) n;
        }
        std::fclose(fp);
        if (!ok) throw std::runtime_error("MeanFluxFile: cannot read " + fname);
        init();
    }

    double operator()(double z) const {
        const size_t n = x_.size();
        if (z < x_[0]) return eval(0, x_[0]) + (z - x_[0]) * slope(0, x_[0]);
        if (z > x_[n - 1]) return eval(n - 2, x_[n - 1]) + (z - x_[n - 1]) * slope(n - 2, x_[n - 1]);
        return eval(interval(z), z);
    }

private:
    std::vector<double> x_, y_, m_;   // knots, values, second derivatives

    // second derivatives with M_0 = M_{n-1} = 0 from the tridiagonal system
    //   h_{i-1} M_{i-1} + 2 (h_{i-1} + h_i) M_i + h_i M_{i+1}
    //     = 6 ((y_{i+1} - y_i) / h_i - (y_i - y_{i-1}) / h_{i-1})
    void init() {
        const size_t n = x_.size();
        if (n < 3 || y_.size() != n) throw std::runtime_error("MeanFlux: needs 3 or more points");
        for (size_t i = 1; i < n; ++i)
            if (!(x_[i] > x_[i - 1])) throw std::runtime_error("MeanFlux: z not increasing");
        m_.assign(n, 0.0);
        const size_t k = n - 2;
        std::vector<double> diag(k), upper(k), rhs(k);
        for (size_t j = 0; j < k; ++j) {
            const size_t i = j + 1;
            const double h0 = x_[i] - x_[i - 1], h1 = x_[i + 1] - x_[i];
            diag[j] = 2.0 * (h0 + h1);
            upper[j] = h1;
            rhs[j] = 6.0 * ((y_[i + 1] - y_[i]) / h1 - (y_[i] - y_[i - 1]) / h0);
        }
        for (size_t j = 1; j < k; ++j) {
            const double f = (x_[j + 1] - x_[j]) / diag[j - 1];
            diag[j] -= f * upper[j - 1];
            rhs[j] -= f * rhs[j - 1];
        }
        m_[k] = rhs[k - 1] / diag[k - 1];
        for (size_t j = k - 1; j-- > 0;) m_[j + 1] = (rhs[j] - upper[j] * m_[j + 2]) / diag[j];
    }
    // i with x_i <= z < x_{i+1} (the last interval at the last knot)
    size_t interval(double z) const {
        size_t lo = 0, hi = x_.size() - 1;
        while (hi - lo > 1) {
            const size_t mid = (lo + hi) / 2;
            if (x_[mid] > z) hi = mid; else lo = mid;
        }
        return lo;
    }
    double eval(size_t i, double z) const {
        const double h = x_[i + 1] - x_[i], t1 = x_[i + 1] - z, t0 = z - x_[i];
        return (m_[i] * t1 * t1 * t1 + m_[i + 1] * t0 * t0 * t0) / (6.0 * h)
             + (y_[i] / h - m_[i] * h / 6.0) * t1 + (y_[i + 1] / h - m_[i + 1] * h / 6.0) * t0;
    }
    double slope(size_t i, double z) const {
        const double h = x_[i + 1] - x_[i], t1 = x_[i + 1] - z, t0 = z - x_[i];
        return (3.0 * m_[i + 1] * t0 * t0 - 3.0 * m_[i] * t1 * t1) / (6.0 * h)
             - (y_[i] / h - m_[i] * h / 6.0) + (y_[i + 1] / h - m_[i + 1] * h / 6.0);
    }
};

// conv::chunkMeanConversion and conv::fullConversion (:94-111): delta =
// F / F-bar - 1 and ivar F-bar^2, F-bar the spectrum's mean flux (over all
// its pixels, masked ones included) or F-bar(z) at each pixel.
inline void convertFluxToDeltaF(Conversion c, const MeanFlux *mean_flux, const double *lambda, double *flux,
                                double *ivar, int size) {
    if (c == Conversion::ChunkMean) {
        double mean = 0;
        for (int i = 0; i < size; ++i) mean += flux[i];
        mean /= size;
        for (int i = 0; i < size; ++i) flux[i] = flux[i] / mean - 1;
        for (int i = 0; i < size; ++i) ivar[i] *= mean * mean;
    } else if (c == Conversion::MeanFluxFile) {
        if (!mean_flux) throw std::runtime_error("convertFluxToDeltaF: no mean flux");
        for (int i = 0; i < size; ++i) {
            const double fbar = (*mean_flux)(lambda[i] / LYA_REST - 1);
            flux[i] = flux[i] / fbar - 1;
            ivar[i] *= fbar * fbar;
        }
    }
}

}  // namespace conv

// The result files of lyspeq's estimator (core/quadratic_estimate.cpp:616-751,
// 797-830; mathtools/matrix_helper.cpp:459-475).  Every number and every line
// a reader parses has the reference's format; the explanatory comments are
// this build's own.
namespace output {

// mxhelp::fprintfMatrix: "nrows ncols", then each row as %14le values
inline void fprintfMatrix(const std::string &fname, const double *a, int nrows, int ncols) {
    std::FILE *f = std::fopen(fname.c_str(), "w");
    if (!f) throw std::runtime_error("cannot write " + fname);
    std::fprintf(f, "%d %d\n", nrows, ncols);
    for (int i = 0; i < nrows; ++i) {
        for (int j = 0; j < ncols; ++j) std::fprintf(f, "%14le ", a[(size_t) i * ncols + j]);
        std::fprintf(f, "\n");
    }
    std::fclose(f);
}

// mxhelp::fscanfMatrix (mathtools/matrix_helper.cpp:477-501): the format
// fprintfMatrix writes
inline std::vector<double> fscanfMatrix(const std::string &fname, int &nrows, int &ncols) {
    std::FILE *f = std::fopen(fname.c_str(), "r");
    if (!f) throw std::runtime_error("cannot read " + fname);
    std::vector<double> a;
    bool ok = std::fscanf(f, "%d %d", &nrows, &ncols) == 2 && nrows > 0 && ncols > 0;
    if (ok) {
        a.resize((size_t) nrows * ncols);
        for (auto &x : a) ok = ok && std::fscanf(f, "%le", &x) == 1;
    }
    std::fclose(f);
    if (!ok) throw std::runtime_error("cannot read a matrix from " + fname);
    return a;
}

// The redshift bin a spectrum counts in, from its median wavelength after the
// redshift cut (OneQSOEstimate::getComputeTimeEst, core/one_qso_estimate.cpp:
// 132-174, and QSOFile::readMinMaxMedRedshift, io/qso_file.cpp:293-313); -1
// for a spectrum the reader drops (S/N cut, empty or short after the cut).
// Index zbin + 1 of the estimator's Z_BIN_COUNTS.
inline int redshiftBinOfFile(const std::string &fname, const Specifics &sp, const Binning &bins) {
    try {
        qio::QSOFile q(fname, qio::Binary);
        q.readParameters();
        if (q.snr < sp.min_snr_cut) return -1;
        q.readData();
        q.cutBoundary(bins.z_lower(), bins.z_upper());
        if (q.realSize() < MIN_PIXELS_IN_FILE) return -1;
        const int n = q.size();
        const double *w = q.wave();
        const double wmed = n % 2 == 0 ? (w[n / 2 - 1] + w[n / 2]) / 2 : w[n / 2];
        return bins.findRedshiftBin(wmed / LYA_REST - 1);
    } catch (std::exception &) {
        return -1;
    }
}

// The same for a spectrum given as arrays (no header, so no S/N cut): the
// pixels inside the redshift range with the masked ends removed.
inline int redshiftBinOfSpectrum(const std::vector<double> &wave, const std::vector<double> &ivar,
                                 const Binning &bins) {
    const double l1 = LYA_REST * (1 + bins.z_lower()), l2 = LYA_REST * (1 + bins.z_upper());
    size_t a = std::lower_bound(wave.begin(), wave.end(), l1) - wave.begin();
    size_t b = std::upper_bound(wave.begin(), wave.end(), l2) - wave.begin();
    while (a < b && !(ivar[a] >= 1e-15)) ++a;
    while (b > a && !(ivar[b - 1] >= 1e-15)) --b;
    int real = 0;
    for (size_t i = a; i < b; ++i) real += ivar[i] >= 1e-15;
    if (b <= a || real < MIN_PIXELS_IN_FILE) return -1;
    const size_t n = b - a;
    const double wmed = n % 2 == 0 ? (wave[a + n / 2 - 1] + wave[a + n / 2]) / 2 : wave[a + n / 2];
    return bins.findRedshiftBin(wmed / LYA_REST - 1);
}

// writeSpectrumEstimates: "Nz Nk", the z-bin counts, then z, k_c, P, error
// per bin (P = fiducial + theta, error = sqrt of the inverse Fisher diagonal)
inline void writeSpectrumEstimates(const std::string &fname, const Binning &bins, const std::vector<int> &zcounts,
                                   const double *theta, const double *pfid, const double *inverse) {
    std::FILE *f = std::fopen(fname.c_str(), "w");
    if (!f) throw std::runtime_error("cannot write " + fname);
    const int nk = bins.nk(), nkz = bins.nkz();
    std::fprintf(f, "%d %d\n", bins.nz(), nk);
    for (int c : zcounts) std::fprintf(f, "%d ", c);
    std::fprintf(f, "\n");
    for (int i = 0; i < nkz; ++i) {
        const int kn = i % nk, zm = i / nk;
        std::fprintf(f, "%.3lf %e %e %e\n", bins.z_centers[zm], (bins.k_edges[kn] + bins.k_edges[kn + 1]) / 2,
                     theta[i] + pfid[i], std::sqrt(inverse[(size_t) (nkz + 1) * i]));
    }
    std::fclose(f);
}

// writeDetailedSpectrumEstimates: comment lines (the settings, the fiducial
// parameters, the damping, "Nz Nk" and the z-bin counts), the column names,
// then per bin z, k1, k2, kc, Pfid, ThetaP, Pest, ErrorP, the Fisher-weighted
// d, b, t and the d, b, t sums before the weighting.
inline void writeDetailedSpectrumEstimates(const std::string &fname, const Binning &bins, const Specifics &sp,
                                           const std::vector<int> &zcounts, bool damped, double damp,
                                           const double *theta, const double *pfid, const double *inverse,
                                           const double *const weighted[3], const double *const sums[3],
                                           bool fisher_optimization) {
    std::FILE *f = std::fopen(fname.c_str(), "w");
    if (!f) throw std::runtime_error("cannot write " + fname);
    std::fprintf(f, "# lyspeq estimate computed by the GB300 engine (lyspeq_gb300)\n");
    std::fprintf(f, "# Fisher optimization: %s\n", fisher_optimization ? "ON" : "OFF");
    std::fprintf(f, "# MaximumForestLength %g\n# DynamicChunkNumber %d\n# ContinuumLogLambdaMargOrder %d\n"
                    "# ContinuumLambdaMargOrder %d\n# TurnOffBaseline %d\n# SmoothNoiseWeights %d\n"
                    "# RedshiftGrowthOn %d\n# UseResoMatrix %d\n",
                 sp.max_forest_length, sp.number_of_chunks, sp.cont_logl_order, sp.cont_l_order,
                 sp.turn_off_sfid ? 1 : 0, sp.smooth_noise_weights, sp.redshift_growth_on ? 1 : 0,
                 sp.use_reso_matrix ? 1 : 0);
    std::fprintf(f, "# Fiducial PD13 power (A, n, alpha, B, beta, lambda):\n");
    for (double v : sp.fiducial) std::fprintf(f, "# %15e\n", v);
    std::fprintf(f, "# Columns: z bin centre; k band lower edge, upper edge, centre [s/km]; fiducial power,\n"
                    "# theta = d - b - t, their sum and sqrt(diag F^-1) [km/s]; Fisher-weighted d, b, t;\n"
                    "# d, b, t before the Fisher weighting.  The counts are of spectra per redshift bin,\n"
                    "# the first and last out of range.\n");
    std::fprintf(f, damped ? "# Damped: True\n" : "# Damped: False\n");
    std::fprintf(f, "# Damping constant: %.3e\n", damp);
    std::fprintf(f, "# %d %d\n# ", bins.nz(), bins.nk());
    for (int c : zcounts) std::fprintf(f, "%d ", c);
    std::fprintf(f, "\n");
    std::fprintf(f, "%5s %14s %14s %14s %14s %14s %14s %14s %14s %14s %14s %14s %14s %14s\n", "z", "k1", "k2", "kc",
                 "Pfid", "ThetaP", "Pest", "ErrorP", "d", "b", "t", "Fd", "Fb", "Ft");
    const int nk = bins.nk(), nkz = bins.nkz();
    for (int i = 0; i < nkz; ++i) {
        const int kn = i % nk, zm = i / nk;
        const double k1 = bins.k_edges[kn], k2 = bins.k_edges[kn + 1];
        std::fprintf(f, "%5.3lf %14e %14e %14e %14e %14e %14e %14e %14e %14e %14e %14e %14e %14e\n",
                     bins.z_centers[zm], k1, k2, (k1 + k2) / 2, pfid[i], theta[i], pfid[i] + theta[i],
                     std::sqrt(inverse[(size_t) (nkz + 1) * i]), weighted[0][i], weighted[1][i], weighted[2][i],
                     sums[0][i], sums[1][i], sums[2][i]);
    }
    std::fclose(f);
}

}  // namespace output

class OneDQuadraticPowerEstimate;

// One chunk of a spectrum in the estimator's batch (Chunk).
class Chunk {
public:
    int fisher_index_start = 0, N_Q_MATRICES = 0;
    int ZBIN_LOW = 0, ZBIN_UPP = 0, KBIN_UPP = 0, RES_INDEX = 0;
    // filled by oneQSOiteration, or by OneDQuadraticPowerEstimate::fetchResults
    std::vector<std::unique_ptr<double[]>> dbt_estimate_before_fisher_vector;
    std::unique_ptr<double[]> fisher_matrix;   // N_Q x N_Q, upper triangle, not halved
    int status = LQG_CHUNK_OK;

    Chunk() = default;
    // Chunk::Chunk (core/chunk_estimate.cpp:141-257): pixels [i1, i2) of a read
    // file join the current estimator's batch; a chunk the reference rejects
    // throws std::runtime_error (short, no table, out of the redshift range)
    Chunk(const qio::QSOFile &qmaster, int i1, int i2);

    // Chunk::oneQSOiteration (core/chunk_estimate.cpp:837-914): this chunk's
    // d, b, t and Fisher matrix at theta = ps_estimate (TOTAL_KZ_BINS), added
    // to dbt_sum_vector (3 x TOTAL_KZ_BINS) at fisher_index_start and to
    // fisher_sum (TOTAL_KZ_BINS^2, upper triangle, not halved) at diagonal
    // offset fisher_index_start.  The first call for a theta computes every
    // chunk of the batch in one GPU iteration; a failed chunk throws.
    void oneQSOiteration(const double *ps_estimate, std::vector<std::unique_ptr<double[]>> &dbt_sum_vector,
                         double *fisher_sum);

    int size() const { return n_pix; }

private:
    friend class OneDQuadraticPowerEstimate;
    int n_pix = 0, batch_index = -1;
    OneDQuadraticPowerEstimate *owner = nullptr;
};

// One spectrum cut into chunks (OneQSOEstimate).
class OneQSOEstimate {
public:
    std::string fname_qso;
    std::vector<std::unique_ptr<Chunk>> chunks;

    OneQSOEstimate() = default;
    // OneQSOEstimate::OneQSOEstimate (core/one_qso_estimate.cpp:52-121): reads
    // the binary file, masks outliers, cuts to the redshift range, drops a
    // short file, decides the chunk boundaries and makes one Chunk per range;
    // a rejected file or chunk is logged and skipped, as the reference does.
    explicit OneQSOEstimate(const std::string &f_qso);

    // OneQSOEstimate::oneQSOiteration (core/one_qso_estimate.cpp:176-197):
    // every chunk's oneQSOiteration; a chunk that fails is dropped.
    void oneQSOiteration(const double *ps_estimate, std::vector<std::unique_ptr<double[]>> &dbt_sum_vector,
                         double *fisher_sum);

    // OneQSOEstimate::_readQsoFile (core/one_qso_estimate.cpp:52-100) on an
    // opened binary file: header, S/N cut, data, flux -> delta (mean_flux:
    // the estimator's F-bar(z) when Specifics names a MeanFluxFile), outlier
    // mask, redshift cut, short-file check.  Throws std::runtime_error where
    // the reference drops the file; returns the number of outliers masked.
    static int readQsoFile(qio::QSOFile &q, const Specifics &sp, double z_lower, double z_upper,
                           const conv::MeanFlux *mean_flux) {
        q.readParameters();
        if (q.snr < sp.min_snr_cut) throw std::runtime_error("OneQSOEstimate::_readQsoFile::Low SNR");
        q.readData();
        conv::convertFluxToDeltaF(conv::conversion(sp), mean_flux, q.wave(), q.delta(), q.ivar(), q.size());
        const int nout = q.maskOutliers();
        q.cutBoundary(z_lower, z_upper);
        if (q.realSize() < MIN_PIXELS_IN_FILE) throw std::runtime_error("OneQSOEstimate::_readQsoFile::Short file");
        return nout;
    }

    // OneQSOEstimate::decideIndices, core/one_qso_estimate.cpp:17-50
    static std::vector<int> decideIndices(int size, const double *wave, const Specifics &sp) {
        std::vector<double> vel(size);
        for (int i = 0; i < size; ++i) vel[i] = SPEED_OF_LIGHT * std::log(wave[i] / wave[0]);
        double vmax = vel[size - 1];
        int nchunks = 1;
        if (sp.number_of_chunks > 1) {
            nchunks += (int) (vmax / sp.max_forest_length_v());
            vmax = std::min(sp.max_forest_length_v(), vmax / nchunks);
        }
        std::vector<int> idx{0};
        int vl = 0;
        for (int i = 0; i < nchunks; ++i) {
            int jj = (int) (std::upper_bound(vel.begin() + vl, vel.end(), vmax) - vel.begin());
            idx.push_back(jj);
            if (jj == size) break;
            vl = jj;
            const double v0 = vel[vl];
            for (int k = vl; k < size; ++k) vel[k] -= v0;
        }
        return idx;
    }
};

class OneDQuadraticPowerEstimate {
public:
    // 3 x TOTAL_KZ_BINS
    std::vector<std::unique_ptr<double[]>> dbt_estimate_sum_before_fisher_vector,
        dbt_estimate_fisher_weighted_vector;
    // TOTAL_KZ_BINS
    std::unique_ptr<double[]> current_power_estimate_vector, previous_power_estimate_vector, powerspectra_fits;
    // TOTAL_KZ_BINS^2 (fisher_matrix_sum as downloaded: upper triangle, not
    // halved; fisher_matrix_halved: halved and symmetric, as the reference
    // holds it after an iteration)
    std::unique_ptr<double[]> fisher_matrix_sum, inverse_fisher_matrix_sum, solver_invfisher_matrix;
    std::vector<double> fisher_matrix_halved;
    // bootstrap(): mean of the realizations, covariance / 4, F^-1 (covariance / 4) F^-T
    std::vector<double> bootstrap_mean, bootstrap_fisher_covariance, bootstrap_covariance;
    int bootstrap_valid = 0;
    std::vector<std::unique_ptr<OneQSOEstimate>> local_queue;
    int damped = 0, dof = 0;
    double damp = 0;

    std::function<void(const std::string &)> log = [](const std::string &) {};

    OneDQuadraticPowerEstimate(const Binning &bins, const SQGrid &grid, const std::vector<SQTable> &tables,
                               const Specifics &sp, int device = 0)
        : bins_(bins), sp_(sp) {
        // conv::readConversion: the mean-flux file is read once, up front
        if (conv::conversion(sp) == conv::Conversion::MeanFluxFile)
            mean_flux_ = std::make_unique<conv::MeanFlux>(sp.mean_flux_file);
        nkz_ = bins.nkz();
        // _readPrecomputedFisher (core/quadratic_estimate.cpp:854-863)
        if (!sp.precomputed_fisher_file.empty()) {
            int nr = 0, nc = 0;
            precomputed_fisher_ = output::fscanfMatrix(sp.precomputed_fisher_file, nr, nc);
            if (nr != nkz_ || nc != nkz_)
                throw std::invalid_argument("Precomputed Fisher matrix does not have correct number of rows or columns.");
        }
        std::vector<int> r;
        std::vector<double> dv, deriv, signal;
        for (const auto &t : tables) {
            r.push_back(t.r_fwhm);
            dv.push_back(t.dv);
            deriv.insert(deriv.end(), t.deriv.begin(), t.deriv.end());
            signal.insert(signal.end(), t.signal.begin(), t.signal.end());
        }
        lqg_bins b{bins.nk(), bins.nz(), bins.k_edges.data(), bins.z_centers.data(), bins.z_bin_width,
                   bins.triangular ? 1 : 0};
        lqg_tables tb{(int) tables.size(), r.data(), dv.data(), grid.nv, grid.v_length, grid.nzp,
                      deriv.data(), sp.turn_off_sfid ? nullptr : signal.data()};
        lqg_opts o{sp.max_forest_length_v(), sp.max_mean_pixel_size, sp.cont_logl_order, sp.cont_l_order,
                   sp.turn_off_sfid ? 1 : 0, sp.precomputed_fisher || !sp.precomputed_fisher_file.empty() ? 1 : 0, 0,
                   sp.smooth_noise_weights,
                   sp.redshift_growth_on ? 1 : 0, sp.fiducial[3]};
        lqg_ctx *c = nullptr;
        if (lqg_ctx_create(&c, &b, &tb, &o, device) != LQG_OK)
            throw std::runtime_error("lqg_ctx_create failed (tables, binning or CUDA device)");
        ctx_.reset(c);
#ifdef FISHER_OPTIMIZATION
        // the caller's build option (./configure --enable-fisher-optimization)
        lqg_set_fisher_optimization(c, 1);
#endif
        for (int i = 0; i < 3; ++i) {
            dbt_estimate_sum_before_fisher_vector.emplace_back(new double[nkz_]());
            dbt_estimate_fisher_weighted_vector.emplace_back(new double[nkz_]());
        }
        current_power_estimate_vector.reset(new double[nkz_]());
        previous_power_estimate_vector.reset(new double[nkz_]());
        powerspectra_fits.reset(new double[nkz_]());
        fisher_matrix_halved.assign((size_t) nkz_ * nkz_, 0.0);
        fisher_matrix_sum.reset(new double[(size_t) nkz_ * nkz_]());
        inverse_fisher_matrix_sum.reset(new double[(size_t) nkz_ * nkz_]());
        solver_invfisher_matrix.reset(new double[(size_t) nkz_ * nkz_]());
        z_bin_counts.assign(bins.nz() + 2, 0);
        current_slot() = this;
    }
    ~OneDQuadraticPowerEstimate() {
        if (current_slot() == this) current_slot() = nullptr;
    }
    OneDQuadraticPowerEstimate(const OneDQuadraticPowerEstimate &) = delete;
    OneDQuadraticPowerEstimate &operator=(const OneDQuadraticPowerEstimate &) = delete;

    // The process's current estimator (the last one constructed): what the
    // reference-signature constructors of OneQSOEstimate and Chunk use.
    static OneDQuadraticPowerEstimate *current() { return current_slot(); }

    // Precision of the batched iterations that Chunk::oneQSOiteration runs.
    Precision chunk_precision = Precision::FP64;

    const Binning &binning() const { return bins_; }
    const Specifics &specifics() const { return sp_; }
    // F-bar(z) of the MeanFluxFile the specifics name (else null)
    const conv::MeanFlux *meanFlux() const { return mean_flux_.get(); }

    // Z_BIN_COUNTS: spectra per redshift bin, index zbin + 1 (0 and
    // NUMBER_OF_Z_BINS + 1: out of range or dropped), counted as each
    // OneQSOEstimate is made
    std::vector<int> z_bin_counts;
    void countSpectrum(int zbin) { ++z_bin_counts[std::max(-1, std::min(zbin, bins_.nz())) + 1]; }

    std::vector<double> fiducialPowers() const {
        std::vector<double> p(nkz_);
        for (int i = 0; i < nkz_; ++i) p[i] = powerSpectrumFiducial(i);
        return p;
    }
    // writeSpectrumEstimates (core/quadratic_estimate.cpp:624-656)
    void writeSpectrumEstimates(const std::string &fname) const {
        output::writeSpectrumEstimates(fname, bins_, z_bin_counts, current_power_estimate_vector.get(),
                                       fiducialPowers().data(), inverse_fisher_matrix_sum.get());
    }
    // writeDetailedSpectrumEstimates (:658-751)
    void writeDetailedSpectrumEstimates(const std::string &fname) const {
        const double *w[3] = {dbt_estimate_fisher_weighted_vector[0].get(), dbt_estimate_fisher_weighted_vector[1].get(),
                              dbt_estimate_fisher_weighted_vector[2].get()};
        const double *d[3] = {dbt_estimate_sum_before_fisher_vector[0].get(),
                              dbt_estimate_sum_before_fisher_vector[1].get(),
                              dbt_estimate_sum_before_fisher_vector[2].get()};
#ifdef FISHER_OPTIMIZATION
        const bool fopt = true;
#else
        const bool fopt = false;
#endif
        output::writeDetailedSpectrumEstimates(fname, bins_, sp_, z_bin_counts, damped != 0, damp,
                                               current_power_estimate_vector.get(), fiducialPowers().data(),
                                               inverse_fisher_matrix_sum.get(), w, d, fopt);
    }
    // writeFisherMatrix (:616-622): the halved, symmetric sum
    void writeFisherMatrix(const std::string &fname) const {
        output::fprintfMatrix(fname, fisher_matrix_halved.data(), nkz_, nkz_);
    }
    // iterationOutput (:797-830): the detailed estimate and the Fisher, inverse
    // Fisher and solver matrices of iteration it (1-based), under
    // OutputDir/OutputFileBase
    void iterationOutput(int it) const {
        const std::string base = sp_.output_dir + "/" + sp_.output_file_base + "_it" + std::to_string(it);
        writeDetailedSpectrumEstimates(base + "_quadratic_power_estimate_detailed.txt");
        writeFisherMatrix(base + "_fisher_matrix.txt");
        output::fprintfMatrix(base + "_inversefisher_matrix.txt", inverse_fisher_matrix_sum.get(), nkz_, nkz_);
        output::fprintfMatrix(base + "_solver_invfishermatrix.txt", solver_invfisher_matrix.get(), nkz_, nkz_);
    }
    int totalKZBins() const { return nkz_; }

    int numberOfChunks() const { return lqg_batch_size(ctx_.get()); }

    // OneQSOEstimate(fname): cleaning of the spectrum (QSOFile::maskOutliers,
    // io/qso_file.cpp:189-230; cutBoundary :159-187; _cutMaskedBoundary
    // :139-157), decideIndices, then one Chunk per pixel range.  A spectrum or
    // chunk the reference rejects is skipped and logged.
    OneQSOEstimate &addQSO(const QSOSpectrum &q) {
        auto est = std::make_unique<OneQSOEstimate>();
        std::vector<double> w = q.wave, d = q.delta, iv = q.ivar;
        const size_t n0 = w.size();
        if (d.size() != n0 || iv.size() != n0) throw std::invalid_argument("QSOSpectrum arrays differ in size");
        countSpectrum(output::redshiftBinOfSpectrum(w, iv, bins_));
        for (auto &x : iv)
            if (x < 1e-15) x = 0;
        maskOutliers(w, d, iv, 5.0);
        const double l1 = LYA_REST * (1 + bins_.z_lower()), l2 = LYA_REST * (1 + bins_.z_upper());
        size_t a = std::lower_bound(w.begin(), w.end(), l1) - w.begin();
        size_t b = std::upper_bound(w.begin(), w.end(), l2) - w.begin();
        while (a < b && iv[a] == 0) ++a;
        while (b > a && iv[b - 1] == 0) --b;
        const int real = (int) std::count_if(iv.begin() + a, iv.begin() + b, [](double x) { return x != 0; });
        if (b <= a || real < MIN_PIXELS_IN_FILE) {
            log("spectrum skipped: short or empty after the redshift and mask cuts");
            local_queue.push_back(std::move(est));
            return *local_queue.back();
        }
        const int size = (int) (b - a);
        std::vector<int> idx = OneQSOEstimate::decideIndices(size, w.data() + a, sp_);
        const int nch = (int) idx.size() - 1;
        std::vector<int64_t> offs(nch + 1, 0);
        for (int i = 0; i < nch; ++i) offs[i + 1] = offs[i] + (idx[i + 1] - idx[i]);
        std::vector<int> rr(nch, q.r_fwhm), st(nch, 0);
        const int before = lqg_batch_size(ctx_.get());
        if (sp_.use_reso_matrix) {
            // Resolution matrix as OneQSOEstimate::_readQsoFile prepares it
            // (core/one_qso_estimate.cpp:75-89): smoothing, deconvolution and
            // oversampling on the whole spectrum, then one row (or column of
            // diagonals) per pixel
            const int nd = q.ndiags;
            if (nd < 1 || q.resomat.size() != (size_t) nd * n0)
                throw std::invalid_argument("QSOSpectrum resomat must hold ndiags x n values");
            std::vector<double> vals = q.resomat;
            if (sp_.smooth_resolution_matrix && sp_.smooth_noise_weights >= 0)
                check(lqg_resomat_smooth((int) n0, nd, vals.data(), sp_.smooth_noise_weights), "lqg_resomat_smooth");
            if (sp_.resomat_deconvolution_m > 0)
                check(lqg_resomat_deconvolve((int) n0, nd, vals.data(), sp_.resomat_deconvolution_m),
                      "lqg_resomat_deconvolve");
            int nelem = nd;
            std::vector<double> per_pixel;
            if (sp_.oversampling > 0) {
                nelem = 2 * (nd / 2) * sp_.oversampling + 1;
                std::vector<double> dl(n0 - 1);
                for (size_t i = 0; i + 1 < n0; ++i) dl[i] = q.wave[i + 1] - q.wave[i];
                std::sort(dl.begin(), dl.end());
                const size_t m = dl.size();
                const double dlambda = (m % 2 == 0) ? (dl[m / 2 - 1] + dl[m / 2]) / 2 : dl[m / 2];
                per_pixel.resize(n0 * nelem);
                check(lqg_resomat_oversample((int) n0, nd, vals.data(), sp_.oversampling, dlambda,
                                             per_pixel.data()),
                      "lqg_resomat_oversample");
            } else {
                per_pixel.resize(n0 * nd);
                for (size_t c = 0; c < n0; ++c)
                    for (int k = 0; k < nd; ++k) per_pixel[c * nd + k] = vals[(size_t) k * n0 + c];
            }
            check(lqg_batch_add_reso(ctx_.get(), nch, offs.data(), w.data() + a, d.data() + a, iv.data() + a,
                                     sp_.oversampling, nelem, per_pixel.data() + a * nelem, st.data()),
                  "lqg_batch_add_reso");
        } else {
            check(lqg_batch_add(ctx_.get(), nch, offs.data(), w.data() + a, d.data() + a, iv.data() + a,
                                rr.data(), st.data()),
                  "lqg_batch_add");
        }
        int next = before;
        for (int i = 0; i < nch; ++i) {
            if (st[i] != LQG_CHUNK_OK) {
                log("chunk skipped: status " + std::to_string(st[i]));
                continue;
            }
            auto ch = std::make_unique<Chunk>();
            int info[8];
            check(lqg_chunk_info(ctx_.get(), next, info), "lqg_chunk_info");
            ch->n_pix = info[0];
            ch->fisher_index_start = info[1];
            ch->N_Q_MATRICES = info[2];
            ch->KBIN_UPP = info[3];
            ch->RES_INDEX = info[4];
            ch->ZBIN_LOW = info[5];
            ch->ZBIN_UPP = info[6];
            ch->batch_index = next++;
            ch->owner = this;
            est->chunks.push_back(std::move(ch));
        }
        local_queue.push_back(std::move(est));
        return *local_queue.back();
    }

    // iterate() (core/quadratic_estimate.cpp:398-528): per iteration every
    // chunk's d, b, t and Fisher matrix (one batched lqg_nr_iteration with
    // powerspectra_fits as the offset from the fiducial), the sums,
    // invertTotalFisherMatrix and computePowerSpectrumEstimates; then
    // hasConverged, and unless done the smoothing of the estimate into the
    // next powerspectra_fits.  Returns the number of iterations run.
    int iterate(int number_of_iterations = 1, Precision precision = Precision::FP64) {
        int it = 0;
        for (it = 1; it <= number_of_iterations; ++it) {
            check(lqg_nr_iteration(ctx_.get(), powerspectra_fits.get(), (int) precision), "lqg_nr_iteration");
            check(lqg_download(ctx_.get(), dbt_estimate_sum_before_fisher_vector[0].get(),
                               dbt_estimate_sum_before_fisher_vector[1].get(),
                               dbt_estimate_sum_before_fisher_vector[2].get(), fisher_matrix_sum.get(), nullptr),
                  "lqg_download");
            // PrecomputedFisher in place of the sum (:478-483); as the unhalved
            // sum the solve takes, which it halves back exactly
            for (size_t e = 0; e < precomputed_fisher_.size(); ++e) fisher_matrix_sum[e] = 2.0 * precomputed_fisher_[e];
            std::copy(current_power_estimate_vector.get(), current_power_estimate_vector.get() + nkz_,
                      previous_power_estimate_vector.get());
            invertTotalFisherMatrix();
            if (!sp_.output_file_base.empty()) iterationOutput(it);
            if (hasConverged() || it == number_of_iterations) break;
            smoothPowerSpectra();
        }
        return std::min(it, number_of_iterations);
    }

    // P_fid(k_c, z_c) of bin i_kz (powerSpectrumFiducial, core/quadratic_estimate.cpp;
    // PD13 fit, core/fiducial_cosmology.cpp:273-282), 0 with TurnOffBaseline
    double powerSpectrumFiducial(int i_kz) const {
        if (sp_.turn_off_sfid) return 0;   // no fiducial signal in C, none in the estimate
        const int kn = i_kz % bins_.nk(), zm = i_kz / bins_.nk();
        return fiducialPowerPD13((bins_.k_edges[kn] + bins_.k_edges[kn + 1]) / 2, bins_.z_centers[zm], sp_.fiducial);
    }

    // hasConverged (core/quadratic_estimate.cpp:548-614): with
    // dp = previous - current (left in previous_power_estimate_vector),
    // sqrt(sum dp^2 / diag(F^-1) / dof) or sqrt(|dp^T F dp| / dof) below
    // ChiSqConvergence.
    bool hasConverged() {
        double *dp = previous_power_estimate_vector.get();
        for (int i = 0; i < nkz_; ++i) dp[i] -= current_power_estimate_vector[i];
        double r = 0, rfull = 0;
        for (int i = 0; i < nkz_; ++i) {
            const double e = inverse_fisher_matrix_sum[(size_t) (nkz_ + 1) * i];
            if (e > 0) r += dp[i] * dp[i] / e;
        }
        const std::vector<double> &fh = fisher_matrix_halved;
        for (int i = 0; i < nkz_; ++i) {
            double s = 0;
            for (int j = 0; j < nkz_; ++j) s += fh[(size_t) i * nkz_ + j] * dp[j];
            rfull += dp[i] * s;
        }
        r = std::sqrt(r / dof);
        rfull = std::sqrt(std::fabs(rfull) / dof);
        return r < sp_.chisq_convergence || rfull < sp_.chisq_convergence;
    }

    // _smoothPowerSpectra (core/quadratic_estimate.cpp:353-396): the estimate
    // as writeSpectrumEstimates prints it, the smoothing command, and its
    // output minus P_fid as the next powerspectra_fits.
    void smoothPowerSpectra() {
        const std::string in = sp_.tmp_folder + "/tmp-power-0.txt", out = sp_.tmp_folder + "/tmp-smooth-0.txt";
        writeSpectrumEstimates(in);
        const std::string cmd = sp_.smoothing_command + " " + in + " " + out + (sp_.smooth_logk_logp ? " --interp_log" : "");
        if (std::system(cmd.c_str()) != 0) throw std::runtime_error("smoothing error: " + cmd);
        FILE *g = std::fopen(out.c_str(), "r");
        if (!g) throw std::runtime_error("cannot read " + out);
        for (int i = 0; i < nkz_; ++i) {
            if (std::fscanf(g, "%le\n", &powerspectra_fits[i]) != 1) {
                std::fclose(g);
                throw std::runtime_error("Reading fit power values from " + out);
            }
            powerspectra_fits[i] -= powerSpectrumFiducial(i);
        }
        std::fclose(g);
        std::remove(in.c_str());
        std::remove(out.c_str());
    }

    // PoissonBootstrapper after the last iteration (core/quadratic_estimate.cpp:536-545)
    // over this estimator's spectra.  FastBootstrap (the default): bootstrap_mean,
    // bootstrap_fisher_covariance (covariance / 4) and bootstrap_covariance
    // (F^-1 (covariance / 4) F^-T).  FastBootstrap 0 (fast = false): a Fisher
    // solve per realization; bootstrap_mean and bootstrap_covariance of the
    // solved realizations, bootstrap_valid of them valid.
    void bootstrap(int number_of_boots, unsigned long long seed = 0, bool fast = true) {
        std::vector<int> off(1, 0);
        for (const auto &q : local_queue) off.push_back(off.back() + (int) q->chunks.size());
        bootstrap_mean.assign(nkz_, 0.0);
        bootstrap_covariance.assign((size_t) nkz_ * nkz_, 0.0);
        bootstrap_fisher_covariance.assign((size_t) nkz_ * nkz_, 0.0);
        if (!fast) {
            check(lqg_bootstrap_complete(ctx_.get(), (int) local_queue.size(), off.data(), number_of_boots, seed,
                                         bootstrap_mean.data(), bootstrap_covariance.data(), nullptr,
                                         &bootstrap_valid),
                  "lqg_bootstrap_complete");
            return;
        }
        check(lqg_bootstrap(ctx_.get(), (int) local_queue.size(), off.data(), number_of_boots, seed,
                            solver_invfisher_matrix.get(), bootstrap_mean.data(), bootstrap_covariance.data(),
                            bootstrap_fisher_covariance.data(), nullptr),
              "lqg_bootstrap");
        bootstrap_valid = number_of_boots;
    }

    // invertTotalFisherMatrix + computePowerSpectrumEstimates
    // (core/quadratic_estimate.cpp:261-318): F/2, stableInvertSym, theta.
    void invertTotalFisherMatrix() {
        std::vector<double> dbt(3 * (size_t) nkz_), w(3 * (size_t) nkz_), fh((size_t) nkz_ * nkz_);
        for (int i = 0; i < 3; ++i)
            std::copy(dbt_estimate_sum_before_fisher_vector[i].get(),
                      dbt_estimate_sum_before_fisher_vector[i].get() + nkz_, dbt.begin() + (size_t) i * nkz_);
        int rc = lqg_fisher_solve(ctx_.get(), fisher_matrix_sum.get(), dbt.data(), fh.data(),
                                  solver_invfisher_matrix.get(), inverse_fisher_matrix_sum.get(), w.data(),
                                  current_power_estimate_vector.get(), &damped, &dof, &damp);
        if (rc != LQG_OK) throw std::runtime_error(std::string("Fisher matrix inversion: ") + lqg_last_error(ctx_.get()));
        fisher_matrix_halved = fh;
        for (int i = 0; i < 3; ++i)
            std::copy(w.begin() + (size_t) i * nkz_, w.begin() + (size_t) (i + 1) * nkz_,
                      dbt_estimate_fisher_weighted_vector[i].get());
    }

    // Copies every chunk's own results of the last iteration into its
    // dbt_estimate_before_fisher_vector and fisher_matrix members.
    void fetchResults() {
        for (auto &q : local_queue)
            for (auto &ch : q->chunks) {
                const int nq = ch->N_Q_MATRICES;
                ch->dbt_estimate_before_fisher_vector.clear();
                for (int i = 0; i < 3; ++i) ch->dbt_estimate_before_fisher_vector.emplace_back(new double[nq]());
                ch->fisher_matrix.reset(new double[(size_t) nq * nq]());
                check(lqg_chunk_result(ctx_.get(), ch->batch_index, ch->dbt_estimate_before_fisher_vector[0].get(),
                                       ch->dbt_estimate_before_fisher_vector[1].get(),
                                       ch->dbt_estimate_before_fisher_vector[2].get(), ch->fisher_matrix.get()),
                      "lqg_chunk_result");
            }
        std::vector<int> st(numberOfChunks());
        if (!st.empty()) {
            check(lqg_download(ctx_.get(), nullptr, nullptr, nullptr, nullptr, st.data()), "lqg_download");
            for (auto &q : local_queue)
                for (auto &ch : q->chunks) ch->status = st[ch->batch_index];
        }
    }

    // lqg_autotune on the current batch (the per-size plan of Precision::MixedAuto)
    void autotune(double max_rel_err = 1e-5, int max_chunks = 48, int flags = 0) {
        check(lqg_autotune(ctx_.get(), max_rel_err, max_chunks, flags), "lqg_autotune");
    }
    // The table as text, one line "ld form drain gram_k pair" per padded size
    void saveTuning(const std::string &path) const {
        const int n = lqg_tuning_get(ctx_.get(), nullptr, 0);
        std::vector<int> e(LQG_TUNING_FIELDS * (size_t) std::max(n, 1));
        lqg_tuning_get(ctx_.get(), e.data(), n);
        std::FILE *f = std::fopen(path.c_str(), "w");
        if (!f) throw std::runtime_error("cannot write " + path);
        for (int k = 0; k < n; ++k) {
            const int *r = e.data() + LQG_TUNING_FIELDS * k;
            std::fprintf(f, "%d %d %d %d %d\n", r[0], r[1], r[2], r[3], r[4]);
        }
        std::fclose(f);
    }
    void loadTuning(const std::string &path) {
        std::FILE *f = std::fopen(path.c_str(), "r");
        if (!f) throw std::runtime_error("cannot read " + path);
        std::vector<int> e;
        int v[LQG_TUNING_FIELDS];
        while (std::fscanf(f, "%d %d %d %d %d", &v[0], &v[1], &v[2], &v[3], &v[4]) == LQG_TUNING_FIELDS)
            e.insert(e.end(), v, v + LQG_TUNING_FIELDS);
        std::fclose(f);
        check(lqg_tuning_set(ctx_.get(), e.data(), (int) e.size() / LQG_TUNING_FIELDS), "lqg_tuning_set");
    }

    // Device time of the last iteration's phases (ms), lqg_last_timings.
    std::vector<double> timings() const {
        std::vector<double> t(8);
        lqg_last_timings(ctx_.get(), t.data(), 8);
        return t;
    }

private:
    friend class Chunk;
    struct CtxDel {
        void operator()(lqg_ctx *c) const { lqg_ctx_destroy(c); }
    };
    std::unique_ptr<lqg_ctx, CtxDel> ctx_;
    Binning bins_;
    Specifics sp_;
    std::unique_ptr<conv::MeanFlux> mean_flux_;
    std::vector<double> precomputed_fisher_;   // PrecomputedFisher (halved, nkz x nkz), else empty
    int nkz_ = 0;
    // the batched iteration behind Chunk::oneQSOiteration: its theta, the
    // batch size it covered and the chunks' statuses
    std::vector<double> batch_theta_;
    int batch_size_done_ = -1;
    std::vector<int> batch_status_;

    static OneDQuadraticPowerEstimate *&current_slot() {
        static OneDQuadraticPowerEstimate *slot = nullptr;
        return slot;
    }

    // One chunk (pixels already cut to the chunk) into the batch; returns its
    // LQG_CHUNK_* status and, when accepted, its lqg_chunk_info.
    int addChunkPixels(const qio::QSOFile &q, int *info, int &index) {
        const int n = q.size();
        int64_t offs[2] = {0, n};
        int r = q.R_fwhm, st = LQG_CHUNK_OK;
        index = lqg_batch_size(ctx_.get());
        check(lqg_batch_add(ctx_.get(), 1, offs, q.wave(), q.delta(), q.ivar(), &r, &st), "lqg_batch_add");
        if (st == LQG_CHUNK_OK) check(lqg_chunk_info(ctx_.get(), index, info), "lqg_chunk_info");
        return st;
    }

    // Runs one iteration of the whole batch at theta unless the last one was
    // at the same theta over the same batch.
    void runBatch(const double *theta) {
        const int nb = lqg_batch_size(ctx_.get());
        bool same = nb == batch_size_done_ && (int) batch_theta_.size() == nkz_;
        for (int i = 0; same && i < nkz_; ++i) same = batch_theta_[i] == (theta ? theta[i] : 0.0);
        if (same) return;
        check(lqg_nr_iteration(ctx_.get(), theta, (int) chunk_precision), "lqg_nr_iteration");
        batch_status_.assign(std::max(nb, 1), 0);
        check(lqg_download(ctx_.get(), nullptr, nullptr, nullptr, nullptr, batch_status_.data()), "lqg_download");
        batch_theta_.assign(nkz_, 0.0);
        if (theta) std::copy(theta, theta + nkz_, batch_theta_.begin());
        batch_size_done_ = nb;
    }

    void check(int rc, const char *what) {
        if (rc != LQG_OK) throw std::runtime_error(std::string(what) + ": " + lqg_last_error(ctx_.get()));
    }

    static double median(std::vector<double> v) {
        std::sort(v.begin(), v.end());
        const size_t n = v.size();
        return n % 2 == 0 ? (v[n / 2 - 1] + v[n / 2]) / 2 : v[n / 2];
    }

    // QSOFile::maskOutliers (io/qso_file.cpp:189-230)
    static void maskOutliers(const std::vector<double> &w, std::vector<double> &d, std::vector<double> &iv,
                             double factor) {
        std::vector<double> tmp;
        for (size_t i = 0; i < d.size(); ++i)
            if (iv[i] != 0) tmp.push_back(d[i]);
        if (tmp.empty()) return;
        const double med = median(tmp);
        for (auto &x : tmp) x = std::fabs(x - med);
        double mad = 1.4826 * (1.0 + 1.0 / std::sqrt((double) tmp.size())) * median(tmp);
        mad = std::max(1.0, mad);
        for (size_t i = 0; i < d.size(); ++i) {
            if (iv[i] == 0) continue;
            const double s = factor * std::max(1.0 / std::sqrt(iv[i]), mad);
            const double fup = std::exp(1.663e-03 * std::pow(w[i] / LYA_REST, 4.107));
            if (d[i] < (-1.0 - s) || d[i] > (fup + s)) {
                d[i] = 0;
                iv[i] = 0;
            }
        }
    }
};

inline Chunk::Chunk(const qio::QSOFile &qmaster, int i1, int i2) {
    OneDQuadraticPowerEstimate *est = OneDQuadraticPowerEstimate::current();
    if (!est) throw std::runtime_error("Chunk: no OneDQuadraticPowerEstimate in this process");
    qio::QSOFile q(qmaster, i1, i2);
    int info[8], index = -1;
    const int st = est->addChunkPixels(q, info, index);
    switch (st) {
    case LQG_CHUNK_OK: break;
    case LQG_CHUNK_SHORT: throw std::runtime_error("Chunk::_copyQSOFile: Short chunk");
    case LQG_CHUNK_NO_TABLE: throw std::out_of_range("SQLookupTable::findSpecResIndex: no table for (R, dv)");
    case LQG_CHUNK_OUT_OF_RANGE: throw std::runtime_error("Chunk::_findRedshiftBin: out of the redshift range");
    default: throw std::runtime_error("Chunk: rejected, status " + std::to_string(st));
    }
    owner = est;
    n_pix = info[0];
    fisher_index_start = info[1];
    N_Q_MATRICES = info[2];
    KBIN_UPP = info[3];
    RES_INDEX = info[4];
    ZBIN_LOW = info[5];
    ZBIN_UPP = info[6];
    batch_index = index;
}

inline void Chunk::oneQSOiteration(const double *ps_estimate, std::vector<std::unique_ptr<double[]>> &dbt_sum_vector,
                                   double *fisher_sum) {
    if (!owner) throw std::runtime_error("Chunk::oneQSOiteration: chunk is not in a batch");
    owner->runBatch(ps_estimate);
    status = owner->batch_status_[batch_index];
    if (status != LQG_CHUNK_OK)
        throw std::runtime_error("Chunk::oneQSOiteration: chunk failed, status " + std::to_string(status));
    const int nq = N_Q_MATRICES, nkz = owner->nkz_;
    dbt_estimate_before_fisher_vector.clear();
    for (int i = 0; i < 3; ++i) dbt_estimate_before_fisher_vector.emplace_back(new double[nq]());
    fisher_matrix.reset(new double[(size_t) nq * nq]());
    owner->check(lqg_chunk_result(owner->ctx_.get(), batch_index, dbt_estimate_before_fisher_vector[0].get(),
                                  dbt_estimate_before_fisher_vector[1].get(),
                                  dbt_estimate_before_fisher_vector[2].get(), fisher_matrix.get()),
                 "lqg_chunk_result");
    // core/chunk_estimate.cpp:893-903: F at diagonal offset (nkz + 1) fis with
    // stride nkz, d, b, t at fis
    const int fis = fisher_index_start;
    for (int i = 0; i < nq; ++i)
        for (int j = 0; j < nq; ++j) fisher_sum[(size_t) (fis + i) * nkz + fis + j] += fisher_matrix[(size_t) i * nq + j];
    for (int k = 0; k < 3; ++k)
        for (int i = 0; i < nq; ++i) dbt_sum_vector[k][fis + i] += dbt_estimate_before_fisher_vector[k][i];
}

inline OneQSOEstimate::OneQSOEstimate(const std::string &f_qso) : fname_qso(f_qso) {
    OneDQuadraticPowerEstimate *est = OneDQuadraticPowerEstimate::current();
    if (!est) throw std::runtime_error("OneQSOEstimate: no OneDQuadraticPowerEstimate in this process");
    const Specifics &sp = est->specifics();
    const Binning &bins = est->binning();
    // Z_BIN_COUNTS, from the estimator's own pass over the file (getComputeTimeEst)
    est->countSpectrum(output::redshiftBinOfFile(f_qso, sp, bins));
    try {
        qio::QSOFile q(f_qso, qio::Binary);
        const int nout = readQsoFile(q, sp, bins.z_lower(), bins.z_upper(), est->meanFlux());
        if (nout > 0) est->log("found " + std::to_string(nout) + " outlier pixels in " + f_qso);
        const std::vector<int> idx = decideIndices(q.size(), q.wave(), sp);
        const int nchunks = (int) idx.size() - 1;
        for (int nc = 0; nc < nchunks; ++nc) {
            try {
                chunks.push_back(std::make_unique<Chunk>(q, idx[nc], idx[nc + 1]));
            } catch (std::exception &e) {
                est->log(std::string(e.what()) + " Skipping chunk " + std::to_string(nc + 1) + "/" +
                         std::to_string(nchunks) + " of " + f_qso);
            }
        }
    } catch (std::exception &e) {
        est->log(std::string(e.what()) + " in " + f_qso);
    }
}

inline void OneQSOEstimate::oneQSOiteration(const double *ps_estimate,
                                            std::vector<std::unique_ptr<double[]>> &dbt_sum_vector,
                                            double *fisher_sum) {
    OneDQuadraticPowerEstimate *est = OneDQuadraticPowerEstimate::current();
    for (auto &ch : chunks) {
        try {
            ch->oneQSOiteration(ps_estimate, dbt_sum_vector, fisher_sum);
        } catch (std::exception &e) {
            if (est) est->log(std::string(e.what()) + " Skipping " + fname_qso);
            ch.reset();
        }
    }
    chunks.erase(std::remove_if(chunks.begin(), chunks.end(), [](const auto &x) { return !x; }), chunks.end());
}

}  // namespace lyspeq_gb300

#endif  // LYSPEQ_API_HPP
