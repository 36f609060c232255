// Noise-weight smoothing of a chunk's ivar (SmoothNoiseWeights) and of a
// resolution matrix's diagonals (SmoothResolutionMatrix), host side.
//
// lyspeq builds the covariance with a smoothed ivar when SmoothNoiseWeights >= 0
// (Chunk::setInvertCovarianceMatrix, core/chunk_estimate.cpp:685-691, calling
// Smoother::smoothIvar, mathtools/smoother.cpp:171-217); the noise matrix of
// the bias traces keeps the raw ivar.  The smoothed array depends only on the
// chunk's own ivar, so it is formed once when the chunk joins a batch and the
// device path reads it wherever the reference reads the smoothed one.
//
// Steps (the reference's, restated):
//   noise variances n_i = 1 / ivar_i (1e15 where ivar_i = 0), sorted; the
//   statistics use the m smallest, those <= 1e3: their median, mean and the
//   scaled median absolute deviation 1.4826 med|n - median|
//   (_findMedianStatistics, :66-81); pixels with
//   ivar < 1 / (median + 3.5 MAD) count as masked;
//   sigmapix = 0: every pixel gets 1 / mean;
//   sigmapix > 0: ivar is padded by 25 cells each side (padArray, :18-26),
//   masked cells (and the pads next to a masked end pixel) are set to
//   1 / mean (_fillMaskedRegion, :84-99), the padded array is inverted to
//   variances and convolved with a normalised 51-tap Gaussian of width
//   sigmapix (_constructFilter, :102-113); the result is inverted back;
//   masked pixels keep their original ivar.
// padArray writes its right-hand pad at cells [n, n + 25) of the padded array,
// i.e. over the last 25 copied pixels, and leaves cells [n + 25, n + 50) at
// zero.  That is kept here: those zeros become infinite variances, so every
// pixel whose window reaches them (the last 25) gets ivar 0, unless the last
// pixel is masked and the fill replaces the zeros.
#include "lqg_internal.cuh"

#include <algorithm>
#include <cmath>
#include <vector>

namespace lqg {

namespace {

constexpr int kHw = 25, kTaps = 2 * kHw + 1;

// stats::medianOfSortedArray (mathtools/stats.cpp:8-16)
double median_sorted(const double *v, int n) {
    return n % 2 == 0 ? (v[n / 2 - 1] + v[n / 2]) / 2 : v[n / 2];
}

}  // namespace

int smooth_ivar(int n, const double *ivar, int sigmapix, double *out) {
    if (n <= 0 || !ivar || !out || sigmapix < 0) return LQG_ERR_ARG;
    std::vector<double> var(n);
    for (int i = 0; i < n; ++i) var[i] = ivar[i] == 0 ? 1e15 : 1.0 / ivar[i];
    std::sort(var.begin(), var.end());
    int m = n;
    while (m > 0 && var[m - 1] > 1e3) --m;
    if (m == 0) {
        // every pixel is noisier than the statistics admit: the reference's
        // median of an empty range is undefined; the ivar is left as it is
        std::copy(ivar, ivar + n, out);
        return LQG_OK;
    }
    const double median = median_sorted(var.data(), m);
    double sum = 0;
    for (int i = 0; i < m; ++i) sum += var[i];
    const double mean_ivar = 1.0 / (sum / m);
    for (int i = 0; i < m; ++i) var[i] = std::fabs(var[i] - median);
    std::sort(var.begin(), var.begin() + m);
    const double mad = 1.4826 * median_sorted(var.data(), m);
    const double cut = 1.0 / (median + 3.5 * mad);
    std::vector<int> masked;
    for (int i = 0; i < n; ++i)
        if (ivar[i] < cut) masked.push_back(i);
    if (sigmapix == 0) {
        std::fill(out, out + n, mean_ivar);
    } else {
        std::vector<double> pad(n + 2 * kHw, 0.0);
        std::copy(ivar, ivar + n, pad.begin() + kHw);
        std::fill(pad.begin(), pad.begin() + kHw, ivar[0]);
        std::fill(pad.begin() + n, pad.begin() + n + kHw, ivar[n - 1]);
        if (!masked.empty()) {
            if (masked.front() == 0) std::fill(pad.begin(), pad.begin() + kHw, mean_ivar);
            for (int i : masked) pad[i + kHw] = mean_ivar;
            if (masked.back() == n - 1) std::fill(pad.end() - kHw, pad.end(), mean_ivar);
        }
        for (double &v : pad) v = 1.0 / v;
        double g[kTaps], gs = 0;
        for (int k = 0; k < kTaps; ++k) {
            const double x = (k - kHw) * 1. / sigmapix;
            g[k] = std::exp(-(x * x) / 2);
            gs += g[k];
        }
        for (double &v : g) v /= gs;
        for (int i = 0; i < n; ++i) {
            double acc = 0;
            for (int k = 0; k < kTaps; ++k) acc += g[k] * pad[i + k];
            out[i] = 1.0 / acc;
        }
    }
    for (int i : masked) out[i] = ivar[i];
    return LQG_OK;
}

// Smoother::smooth1D (mathtools/smoother.cpp:144-168) over `rows` rows of n
// values each (a resolution matrix's diagonals, SmoothResolutionMatrix):
// sigmapix = 0 replaces a row by the mean of its values <= 1e3; sigmapix > 0
// convolves it with the 51-tap Gaussian after the same padding as above
// (left pad the first value, right pad over the last 25 values, zeros past them).
int smooth_rows(int n, int rows, double *values, int sigmapix) {
    if (n <= 0 || rows <= 0 || !values || sigmapix < 0) return LQG_ERR_ARG;
    double g[kTaps], gs = 0;
    for (int k = 0; k < kTaps; ++k) {
        const double x = (k - kHw) * 1. / sigmapix;
        g[k] = sigmapix > 0 ? std::exp(-(x * x) / 2) : 0.0;
        gs += g[k];
    }
    if (sigmapix > 0)
        for (double &v : g) v /= gs;
    std::vector<double> pad(n + 2 * kHw);
    for (int r = 0; r < rows; ++r) {
        double *row = values + (size_t) r * n;
        if (sigmapix == 0) {
            std::vector<double> v(row, row + n);
            std::sort(v.begin(), v.end());
            int m = n;
            while (m > 0 && v[m - 1] > 1e3) --m;
            double sum = 0;
            for (int i = 0; i < m; ++i) sum += v[i];
            std::fill(row, row + n, sum / m);
            continue;
        }
        std::fill(pad.begin(), pad.end(), 0.0);
        std::copy(row, row + n, pad.begin() + kHw);
        std::fill(pad.begin(), pad.begin() + kHw, row[0]);
        std::fill(pad.begin() + n, pad.begin() + n + kHw, row[n - 1]);
        for (int i = 0; i < n; ++i) {
            double acc = 0;
            for (int k = 0; k < kTaps; ++k) acc += g[k] * pad[i + k];
            row[i] = acc;
        }
    }
    return LQG_OK;
}

}  // namespace lqg

extern "C" int lqg_resomat_smooth(int n, int ndiags, double *values, int sigmapix) {
    return lqg::smooth_rows(n, ndiags, values, sigmapix);
}

extern "C" int lqg_smooth_ivar(int n, const double *ivar, int sigmapix, double *out) {
    if (out == ivar) return LQG_ERR_ARG;
    return lqg::smooth_ivar(n, ivar, sigmapix, out);
}
