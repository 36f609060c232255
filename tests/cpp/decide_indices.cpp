// Host-only check of the facade's chunking (OneQSOEstimate::decideIndices in
// include/lyspeq_api.hpp): reads wavelength arrays from a binary file and
// prints, one line per array, the pixel-range boundaries the facade cuts the
// spectrum into.  Input (little-endian): int64 count, then per array: double
// MaximumForestLength, int64 DynamicChunkNumber, int64 n, n doubles (Angstrom).
#include <cstdint>
#include <cstdio>
#include <vector>

#include "lyspeq_api.hpp"

using namespace lyspeq_gb300;

int main(int argc, char **argv) {
    if (argc != 2) return 2;
    FILE *f = std::fopen(argv[1], "rb");
    if (!f) return 2;
    int64_t count = 0;
    if (std::fread(&count, 8, 1, f) != 1) return 2;
    for (int64_t c = 0; c < count; ++c) {
        double mfl = 0;
        int64_t nch = 0, n = 0;
        if (std::fread(&mfl, 8, 1, f) != 1 || std::fread(&nch, 8, 1, f) != 1 || std::fread(&n, 8, 1, f) != 1 ||
            n < 1)
            return 2;
        std::vector<double> w((size_t) n);
        if (std::fread(w.data(), 8, (size_t) n, f) != (size_t) n) return 2;
        Specifics sp;
        sp.max_forest_length = mfl;
        sp.number_of_chunks = (int) nch;
        const std::vector<int> idx = OneQSOEstimate::decideIndices((int) n, w.data(), sp);
        for (size_t i = 0; i < idx.size(); ++i) std::printf(i ? " %d" : "%d", idx[i]);
        std::printf("\n");
    }
    std::fclose(f);
    return 0;
}
