// ref_loader_main.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Driver linked against the reference's own loader (dataset.cu:10-39,
// compiled from the reference sources by oracle/build_ref.sh into
// oracle/_ref/).  It loads a text dataset with the reference's
// importDataset() and writes "<rows> <dim>\n" followed by the row-major
// doubles in binary to the output file, so the tests can compare the
// library's loader and the oracle's restatement with the reference itself.
// The reference's dimension is its compile-time INPUT_DATA_DIM (params.h:4).
#include <cstdio>
#include <cstdlib>
#include <vector>

void importDataset(std::vector<std::vector<double> >* inputVector, char* filename);

int main(int argc, char** argv)
{
    if (argc != 3) {
        std::fprintf(stderr, "usage: %s <dataset.txt> <out.bin>\n", argv[0]);
        return 2;
    }
    std::vector<std::vector<double> > rows;
    importDataset(&rows, argv[1]);
    FILE* f = std::fopen(argv[2], "wb");
    if (!f) return 3;
    unsigned long long n = rows.size();
    unsigned long long dim = n ? rows[0].size() : 0;
    std::fprintf(f, "%llu %llu\n", n, dim);
    for (const auto& r : rows) std::fwrite(r.data(), sizeof(double), r.size(), f);
    std::fclose(f);
    return 0;
}
