// Host-only check of the facade's result files (namespace output and
// fiducialPowerPD13 in include/lyspeq_api.hpp).  Reads an estimate's numbers
// from a binary file, counts the spectra per redshift bin from the files
// themselves, and writes the four files of one iteration under BASE_it1_*.
//
//   write_outputs IN BASE
//
// IN (little-endian; "vec" = int64 n then n doubles): vec k_edges, vec
// z_centers, double dz, vec fiducial (6), double MinimumSnrCut, int64 damped,
// double damp, vec theta, vec pfid, vec inverse (nkz^2), vec weighted (3 nkz),
// vec sums (3 nkz), vec fisher (nkz^2), vec solver (nkz^2), int64 number of
// spectrum files, then per file int64 length and its path.  Reads the Fisher
// file back (output::fscanfMatrix; exit 3 if it differs) and prints the
// fiducial power of every bin (%.17g), one per line.
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "lyspeq_api.hpp"

using namespace lyspeq_gb300;

namespace {
std::FILE *in;
bool ok = true;
int64_t i64() {
    int64_t v = 0;
    ok = ok && std::fread(&v, 8, 1, in) == 1;
    return v;
}
double f64() {
    double v = 0;
    ok = ok && std::fread(&v, 8, 1, in) == 1;
    return v;
}
std::vector<double> vec() {
    const int64_t n = i64();
    std::vector<double> v(ok && n > 0 ? (size_t) n : 0);
    if (!v.empty()) ok = ok && std::fread(v.data(), 8, v.size(), in) == v.size();
    return v;
}
}  // namespace

int main(int argc, char **argv) {
    if (argc != 3) return 2;
    in = std::fopen(argv[1], "rb");
    if (!in) return 2;
    Binning bins;
    bins.k_edges = vec();
    bins.z_centers = vec();
    bins.z_bin_width = f64();
    Specifics sp;
    const std::vector<double> fid = vec();
    if (fid.size() != 6) return 2;
    std::copy(fid.begin(), fid.end(), sp.fiducial);
    sp.min_snr_cut = f64();
    const bool damped = i64() != 0;
    const double damp = f64();
    const std::vector<double> theta = vec(), pfid = vec(), inverse = vec(), weighted = vec(), sums = vec(),
                              fisher = vec(), solver = vec();
    std::vector<int> counts(bins.nz() + 2, 0);
    const int64_t nfiles = i64();
    for (int64_t i = 0; ok && i < nfiles; ++i) {
        std::string path((size_t) i64(), '\0');
        ok = ok && std::fread(&path[0], 1, path.size(), in) == path.size();
        ++counts[output::redshiftBinOfFile(path, sp, bins) + 1];
    }
    std::fclose(in);
    const int nkz = bins.nkz();
    if (!ok || (int) theta.size() != nkz || (int) weighted.size() != 3 * nkz || (int) fisher.size() != nkz * nkz)
        return 2;
    const double *w[3] = {weighted.data(), weighted.data() + nkz, weighted.data() + 2 * nkz};
    const double *d[3] = {sums.data(), sums.data() + nkz, sums.data() + 2 * nkz};
    const std::string base = std::string(argv[2]) + "_it1";
    output::writeDetailedSpectrumEstimates(base + "_quadratic_power_estimate_detailed.txt", bins, sp, counts, damped,
                                           damp, theta.data(), pfid.data(), inverse.data(), w, d, false);
    output::fprintfMatrix(base + "_fisher_matrix.txt", fisher.data(), nkz, nkz);
    output::fprintfMatrix(base + "_inversefisher_matrix.txt", inverse.data(), nkz, nkz);
    output::fprintfMatrix(base + "_solver_invfishermatrix.txt", solver.data(), nkz, nkz);
    // the matrix reader (PrecomputedFisher) reads the Fisher file back to the
    // values it was written from
    int nr = 0, nc = 0;
    const std::vector<double> back = output::fscanfMatrix(base + "_fisher_matrix.txt", nr, nc);
    if (nr != nkz || nc != nkz || back != fisher) return 3;
    for (int i = 0; i < nkz; ++i) {
        const int kn = i % bins.nk(), zm = i / bins.nk();
        std::printf("%.17g\n", fiducialPowerPD13((bins.k_edges[kn] + bins.k_edges[kn + 1]) / 2, bins.z_centers[zm],
                                                 sp.fiducial));
    }
    return 0;
}
