// Oracle driver (test infrastructure).  Links lyspeq's own translation units,
// compiled unmodified from the reference sources, and runs its per-chunk QMLE
// path on every chunk of a config's spectra, then the global Newton-Raphson
// step, dumping every intermediate result in a flat little-endian binary file
// that the tests read.
//
// Set-up follows LyaPowerEstimate.cpp:21-121 (config, bins, specifics,
// conversion, fiducial cosmology, SQ tables, smoother).  Each chunk's
// contribution is obtained from Chunk::oneQSOiteration
// (core/chunk_estimate.cpp:837-914) with zeroed accumulators, so the dump
// holds the per-chunk d, b, t and Fisher exactly as the reference computes
// them.  The global step repeats core/quadratic_estimate.cpp:456-457
// (F *= 0.5, copyUpperToLower), :261-288 (stableInvertSym) and :290-318
// (theta = 0.5 F^-1 (d - b - t)) with the reference's own mxhelp routines.
//
// With --reso, every spectrum X.dat comes with X.dat.rmat, its resolution
// matrix in the reference's DiaMatrix layout (int32 n, int32 ndiags, then
// ndiags x n doubles, diagonal d holding offset ndiags/2 - d, element of
// column c at [d][c]).  The reference reads such matrices only from picca FITS
// files (io/qso_file.cpp:652-677); the driver attaches them to the binary
// spectrum instead and then follows OneQSOEstimate::_readQsoFile
// (core/one_qso_estimate.cpp:52-100) step by step: deconvolution, oversampling,
// boundary cut, chunking by decideIndices and Chunk::Chunk.  The config's
// OversampleRmat and ResoMatDeconvolutionM keys apply;
// specifics::USE_RESOLUTION_MATRIX is switched on after the config is read.
//
// With --boot N the driver then runs lyspeq's Poisson bootstrap over the
// spectra (PoissonBootstrapper, core/bootstrapper.hpp, after
// OneQSOEstimate::collapseBootstrap, as core/quadratic_estimate.cpp:536-545
// does) and dumps its mean, covariance and realizations at full precision.
// The bootstrapper keeps them in private members and writes them to text
// files with 7 digits only, so this one translation unit opens the class's
// private members when it includes the header (the header itself is used
// unmodified).
//
// With --iterate the driver finally runs lyspeq's whole Newton-Raphson loop,
// OneDQuadraticPowerEstimate::iterate() (core/quadratic_estimate.cpp:398-546:
// NumberOfIterations iterations with convergence tests and the smoothing of
// the estimate by the smbivspline.py script between them; the script must be
// on PATH), and dumps the estimator's final state.
//
// Usage: chunk_driver <config> <out.bin> [--no-pixels] [--reso] [--boot N [--boot-complete]] [--iterate]
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "core/chunk_estimate.hpp"
#include "core/fiducial_cosmology.hpp"
#include "core/global_numbers.hpp"
#include "core/one_qso_estimate.hpp"
#include "core/sq_table.hpp"
#include "io/qso_file.hpp"
#include "io/config_file.hpp"
#include "io/io_helper_functions.hpp"
#include "io/logger.hpp"
#include "mathtools/matrix_helper.hpp"
#include "mathtools/smoother.hpp"
#include <algorithm>
#include <random>
#define private public
#define protected public
#include "core/bootstrapper.hpp"
#include "core/quadratic_estimate.hpp"
#undef protected
#undef private

namespace {
void putI(FILE *f, int v) { std::fwrite(&v, sizeof v, 1, f); }
void putD(FILE *f, const double *v, size_t n) { if (n) std::fwrite(v, sizeof(double), n, f); }

// One spectrum with its resolution matrix, read as OneQSOEstimate::_readQsoFile
// does (core/one_qso_estimate.cpp:52-100), the matrix coming from X.rmat.
std::unique_ptr<OneQSOEstimate> read_with_resomat(const std::string &path) {
    auto q = std::make_unique<OneQSOEstimate>();
    try {
        auto qFile = std::make_unique<qio::QSOFile>(path, qio::Binary);
        qFile->readParameters();
        if (qFile->snr < specifics::MIN_SNR_CUT) throw std::runtime_error("Low SNR");
        qFile->readData();
        conv::convertFluxToDeltaF(qFile->wave(), qFile->delta(), qFile->ivar(), qFile->size());
        qFile->maskOutliers();

        FILE *rf = std::fopen((path + ".rmat").c_str(), "rb");
        if (!rf) throw std::runtime_error("missing resolution matrix file");
        int hdr[2] = {0, 0};
        if (std::fread(hdr, sizeof(int), 2, rf) != 2 || hdr[0] != qFile->size()) {
            std::fclose(rf);
            throw std::runtime_error("resolution matrix size mismatch");
        }
        qFile->Rmat = std::make_unique<mxhelp::Resolution>(hdr[0], hdr[1]);
        size_t nval = (size_t) hdr[0] * hdr[1];
        size_t got = std::fread(qFile->Rmat->matrix(), sizeof(double), nval, rf);
        std::fclose(rf);
        if (got != nval) throw std::runtime_error("short resolution matrix file");
        if (process::smoother->isSmoothingOnRmat())
            process::smoother->smooth1D(qFile->Rmat->matrix(), qFile->Rmat->getNCols(),
                                        qFile->Rmat->getNElemPerRow());
        if (specifics::RESOMAT_DECONVOLUTION_M > 0)
            qFile->Rmat->deconvolve(specifics::RESOMAT_DECONVOLUTION_M);
        if (specifics::OVERSAMPLING_FACTOR > 0)
            qFile->Rmat->oversample(specifics::OVERSAMPLING_FACTOR, qFile->dlambda);
        qFile->closeFile();
        qFile->cutBoundary(bins::Z_LOWER_EDGE, bins::Z_UPPER_EDGE);
        if (qFile->realSize() < 100) throw std::runtime_error("Short file");

        std::vector<int> indices = OneQSOEstimate::decideIndices(qFile->size(), qFile->wave());
        for (size_t nc = 0; nc + 1 < indices.size(); ++nc) {
            try {
                q->chunks.push_back(std::make_unique<Chunk>(*qFile, indices[nc], indices[nc + 1]));
            } catch (std::exception &) {
            }
        }
    } catch (std::exception &e) {
        std::fprintf(stderr, "%s: %s\n", path.c_str(), e.what());
    }
    return q;
}
}

int main(int argc, char *argv[]) {
    if (argc < 3) {
        std::fprintf(stderr, "usage: %s <config> <out.bin> [--no-pixels] [--reso]\n", argv[0]);
        return 2;
    }
    bool dump_pixels = true, reso = false;
    int nboots = 0;
    bool nr_loop = false, boot_complete = false;
    for (int a = 3; a < argc; ++a) {
        if (std::strcmp(argv[a], "--iterate") == 0) { nr_loop = true; continue; }
        if (std::strcmp(argv[a], "--no-pixels") == 0) dump_pixels = false;
        else if (std::strcmp(argv[a], "--reso") == 0) reso = true;
        else if (std::strcmp(argv[a], "--boot") == 0 && a + 1 < argc) nboots = std::atoi(argv[++a]);
        else if (std::strcmp(argv[a], "--boot-complete") == 0) boot_complete = true;
    }

    ConfigFile config;
    config.readFile(argv[1]);
    LOG::LOGGER.open(config.get("OutputDir", "."), 0);
    process::readProcess(config);
    bins::readBins(config);
    specifics::readSpecifics(config);
    conv::readConversion(config);
    if (reso) specifics::USE_RESOLUTION_MATRIX = true;
    fidcosmo::readFiducialCosmo(config);

    process::sq_private_table = std::make_unique<SQLookupTable>(config);
    process::sq_private_table->readTables();
    process::updateMemory(-process::sq_private_table->getMaxMemUsage());
    process::smoother = std::make_unique<Smoother>(config);

    // Keys OneDQuadraticPowerEstimate consumes; read here so checkUnusedKeys passes.
    config.getInteger("NumberOfIterations", 1);
    std::string flist = config.get("FileNameList"), findir = config.get("FileInputDir");
    config.get("Targetids2Ignore");
    config.checkUnusedKeys();
    if (findir.back() != '/') findir += '/';

    std::vector<std::string> fpaths;
    ioh::readList(flist.c_str(), fpaths);

    std::vector<std::unique_ptr<OneQSOEstimate>> qsos;
    qsos.reserve(fpaths.size());
    for (auto &fp : fpaths)
        qsos.push_back(reso ? read_with_resomat(findir + fp)
                            : std::make_unique<OneQSOEstimate>(findir + fp));

    glmemory::allocMemory();

    const int nkz = bins::TOTAL_KZ_BINS;
    std::vector<double> ps(nkz, 0.0);          // powerspectra_fits: zero on the first iteration
    std::vector<std::unique_ptr<double[]>> dbt_sum;
    for (int i = 0; i < 3; ++i) dbt_sum.push_back(std::make_unique<double[]>(nkz));
    auto fisher_sum = std::make_unique<double[]>((size_t) nkz * nkz);

    FILE *out = std::fopen(argv[2], "wb");
    if (!out) { std::perror("fopen"); return 1; }
    std::fwrite("LQGREF02", 1, 8, out);
    putI(out, nkz);
    putI(out, bins::NUMBER_OF_K_BANDS);
    putI(out, bins::NUMBER_OF_Z_BINS);
    int nchunks_total = 0;
    for (auto &q : qsos) nchunks_total += (int) q->chunks.size();
    putI(out, nchunks_total);

    double t_chunks = 0;
    for (size_t iq = 0; iq < qsos.size(); ++iq) {
        for (size_t ic = 0; ic < qsos[iq]->chunks.size(); ++ic) {
            Chunk &ch = *qsos[iq]->chunks[ic];
            const int n = ch.size(), nq = ch.N_Q_MATRICES;
            // Copy the chunk's inputs before the iteration: wave is already lambda/LYA_REST.
            std::vector<double> w(ch.qFile->wave(), ch.qFile->wave() + n),
                d(ch.qFile->delta(), ch.qFile->delta() + n),
                iv(ch.qFile->ivar(), ch.qFile->ivar() + n);
            std::vector<double> rm;
            int rm_dia = 0, rm_nelem = 0;
            if (reso && ch.qFile->Rmat) {
                rm.assign(ch.qFile->Rmat->matrix(), ch.qFile->Rmat->matrix() + ch.qFile->Rmat->getSize());
                rm_dia = ch.qFile->Rmat->isDiaMatrix() ? 1 : 0;
                rm_nelem = ch.qFile->Rmat->getNElemPerRow();
            }

            std::vector<std::unique_ptr<double[]>> dbt_local;
            for (int i = 0; i < 3; ++i) dbt_local.push_back(std::make_unique<double[]>(nkz));
            auto fisher_local = std::make_unique<double[]>((size_t) nkz * nkz);

            auto t0 = std::chrono::steady_clock::now();
            ch.oneQSOiteration(ps.data(), dbt_local, fisher_local.get());
            t_chunks += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();

            // A chunk whose inversion threw contributes nothing (chunk_estimate.cpp:905-913).
            int status = 0;
            bool any = false;
            for (int i = 0; i < 3 && !any; ++i)
                for (int k = 0; k < nkz; ++k) if (dbt_local[i][k] != 0) { any = true; break; }
            if (!any) status = 1;

            for (int i = 0; i < 3; ++i)
                for (int k = 0; k < nkz; ++k) dbt_sum[i][k] += dbt_local[i][k];
            for (size_t k = 0; k < (size_t) nkz * nkz; ++k) fisher_sum[k] += fisher_local[k];

            putI(out, (int) iq); putI(out, (int) ic); putI(out, n);
            putI(out, ch.fisher_index_start); putI(out, nq); putI(out, ch.KBIN_UPP);
            putI(out, ch.qFile->R_fwhm); putI(out, status);
            double dv = ch.qFile->dv_kms;
            putD(out, &dv, 1);
            putI(out, dump_pixels ? 1 : 0);
            if (dump_pixels) { putD(out, w.data(), n); putD(out, d.data(), n); putD(out, iv.data(), n); }
            // the chunk's resolution matrix: diagonal (values[ndiags][n]) or
            // oversampled (rows[n][nelem]), as the chunk holds it
            putI(out, (int) rm.size()); putI(out, rm_dia); putI(out, rm_nelem);
            putD(out, rm.data(), rm.size());
            for (int i = 0; i < 3; ++i) putD(out, ch.dbt_estimate_before_fisher_vector[i].get(), nq);
            putD(out, ch.fisher_matrix.get(), (size_t) nq * nq);
        }
    }

    // Global NR step, quadratic_estimate.cpp:456-457 then :261-318.
    auto t1 = std::chrono::steady_clock::now();
    cblas_dscal(nkz * nkz, 0.5, fisher_sum.get(), 1);
    mxhelp::copyUpperToLower(fisher_sum.get(), nkz);
    std::vector<double> fisher_halved(fisher_sum.get(), fisher_sum.get() + (size_t) nkz * nkz);

    auto solver = std::make_unique<double[]>((size_t) nkz * nkz);
    auto invf = std::make_unique<double[]>((size_t) nkz * nkz);
    std::copy_n(fisher_sum.get(), (size_t) nkz * nkz, solver.get());
    int dof = nkz;
    double damp = 0;
    int warn = mxhelp::stableInvertSym(solver, invf, nkz, dof, damp);

    std::vector<std::vector<double>> weighted(3, std::vector<double>(nkz));
    for (int i = 0; i < 3; ++i)
        cblas_dgemv(CblasRowMajor, CblasNoTrans, nkz, nkz, 0.5, solver.get(), nkz,
                    dbt_sum[i].get(), 1, 0, weighted[i].data(), 1);
    std::vector<double> theta(weighted[0]);
    cblas_daxpy(nkz, -1, weighted[1].data(), 1, theta.data(), 1);
    cblas_daxpy(nkz, -1, weighted[2].data(), 1, theta.data(), 1);
    double t_global = std::chrono::duration<double>(std::chrono::steady_clock::now() - t1).count();

    std::fwrite("GLOBAL01", 1, 8, out);
    putD(out, fisher_halved.data(), fisher_halved.size());
    for (int i = 0; i < 3; ++i) putD(out, dbt_sum[i].get(), nkz);
    putD(out, solver.get(), (size_t) nkz * nkz);
    putD(out, invf.get(), (size_t) nkz * nkz);
    putD(out, theta.data(), nkz);
    putI(out, warn); putI(out, dof);
    putD(out, &damp, 1);
    std::vector<double> pfid(nkz);
    for (int i = 0; i < nkz; ++i) {
        int kn, zm;
        bins::getFisherMatrixBinNoFromIndex(i, kn, zm);
        pfid[i] = fidcosmo::fiducialPowerSpectrum(bins::KBAND_CENTERS[kn], bins::ZBIN_CENTERS[zm],
                                                  &fidpd13::FIDUCIAL_PD13_PARAMS);
    }
    putD(out, pfid.data(), nkz);
    putD(out, &t_chunks, 1);
    putD(out, &t_global, 1);
    if (nboots > 0 && boot_complete) {
        // core/quadratic_estimate.cpp:536-545 with FastBootstrap 0: a Cholesky
        // solve of the bootstrapped Fisher matrix per realization
        specifics::FAST_BOOTSTRAP = false;
        PoissonBootstrapper pbooter(nboots, solver.get());
        for (auto &q : qsos) q->collapseBootstrap();
        pbooter.run(qsos);
        std::fwrite("BOOT0002", 1, 8, out);
        putI(out, nboots);
        putI(out, (int) qsos.size());
        putI(out, (int) pbooter.remaining_boots);
        putD(out, pbooter.temppower.get(), nkz);                         // mean of the realizations
        putD(out, pbooter.tempfisher.get(), (size_t) nkz * nkz);         // covariance
        putD(out, pbooter.allpowers.get(), (size_t) nboots * nkz);       // realizations (solved)
    } else if (nboots > 0) {
        // core/quadratic_estimate.cpp:536-545 with FastBootstrap (the default)
        specifics::FAST_BOOTSTRAP = true;
        PoissonBootstrapper pbooter(nboots, solver.get());
        for (auto &q : qsos) q->collapseBootstrap();
        pbooter.run(qsos);
        std::fwrite("BOOT0001", 1, 8, out);
        putI(out, nboots);
        putI(out, (int) qsos.size());
        putD(out, pbooter.temppower.get(), nkz);                         // mean of the realizations
        putD(out, pbooter.tempfisher.get(), (size_t) nkz * nkz);         // F^-1 (cov / 4) F^-T
        putD(out, pbooter.allpowers.get(), (size_t) nboots * nkz);       // realizations
    }
    std::fclose(out);
    glmemory::dealloc();
    if (nr_loop) {
        // LyaPowerEstimate.cpp:109-125 on the set-up above
        OneDQuadraticPowerEstimate qps(config);
        qps.iterate();
        FILE *o2 = std::fopen((std::string(argv[2]) + ".iter").c_str(), "wb");
        if (!o2) { std::perror("fopen"); return 1; }
        std::fwrite("ITER0001", 1, 8, o2);
        putI(o2, nkz);
        putD(o2, qps.current_power_estimate_vector.get(), nkz);
        putD(o2, qps.previous_power_estimate_vector.get(), nkz);
        putD(o2, qps.powerspectra_fits.get(), nkz);
        putD(o2, qps.fisher_matrix_sum.get(), (size_t) nkz * nkz);
        putD(o2, qps.inverse_fisher_matrix_sum.get(), (size_t) nkz * nkz);
        for (int i = 0; i < 3; ++i) putD(o2, qps.dbt_estimate_sum_before_fisher_vector[i].get(), nkz);
        std::fclose(o2);
    }

    std::printf("chunks=%d t_chunks=%.6f s t_global=%.6f s damped=%d\n", nchunks_total, t_chunks,
                t_global, warn);
    return 0;
}
