// Host-only check of the facade's reading of binary spectra
// (OneQSOEstimate::readQsoFile and decideIndices in include/lyspeq_api.hpp),
// flux to delta conversion included: reads each file as the reference's
// OneQSOEstimate does and writes every chunk's pixels as Chunk(QSOFile, i1,
// i2) holds them.
//
//   read_spectra OUT MODE MEANFLUX ZLO ZHI MAXFOREST NCHUNKS FILE...
//
// MODE: 0 delta input, 1 UseChunksMeanFlux, 2 MeanFluxFile (MEANFLUX, else
// "-").  OUT (little-endian): per file int64 number of chunks (-1: the file
// is dropped), then per chunk int64 n and n doubles each of lambda
// (Angstrom), delta and ivar (n = 0: the chunk is masked throughout).
#include <cstdint>
#include <cstdio>
#include <memory>
#include <string>
#include <vector>

#include "lyspeq_api.hpp"

using namespace lyspeq_gb300;

int main(int argc, char **argv) {
    if (argc < 9) return 2;
    std::FILE *out = std::fopen(argv[1], "wb");
    if (!out) return 2;
    const int mode = std::atoi(argv[2]);
    Specifics sp;
    sp.input_is_delta_flux = mode == 0;
    sp.use_chunks_mean_flux = mode == 1;
    if (mode == 2) sp.mean_flux_file = argv[3];
    const double zlo = std::atof(argv[4]), zhi = std::atof(argv[5]);
    sp.max_forest_length = std::atof(argv[6]);
    sp.number_of_chunks = std::atoi(argv[7]);
    std::unique_ptr<conv::MeanFlux> mean_flux;
    if (conv::conversion(sp) == conv::Conversion::MeanFluxFile)
        mean_flux = std::make_unique<conv::MeanFlux>(sp.mean_flux_file);
    auto put = [&](const void *p, size_t bytes) { std::fwrite(p, 1, bytes, out); };
    for (int a = 8; a < argc; ++a) {
        qio::QSOFile q(argv[a], qio::Binary);
        int64_t nchunks = -1;
        try {
            OneQSOEstimate::readQsoFile(q, sp, zlo, zhi, mean_flux.get());
        } catch (std::exception &) {
            put(&nchunks, 8);
            continue;
        }
        const std::vector<int> idx = OneQSOEstimate::decideIndices(q.size(), q.wave(), sp);
        nchunks = (int64_t) idx.size() - 1;
        put(&nchunks, 8);
        for (int64_t c = 0; c < nchunks; ++c) {
            std::unique_ptr<qio::QSOFile> ch;
            try {
                ch = std::make_unique<qio::QSOFile>(q, idx[c], idx[c + 1]);
            } catch (std::exception &) {   // masked throughout: the reference drops it too
                const int64_t zero = 0;
                put(&zero, 8);
                continue;
            }
            const int64_t n = ch->size();
            put(&n, 8);
            put(ch->wave(), 8 * n);
            put(ch->delta(), 8 * n);
            put(ch->ivar(), 8 * n);
        }
    }
    std::fclose(out);
    return 0;
}
