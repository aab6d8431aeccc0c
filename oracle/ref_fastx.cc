// Test infrastructure: runs the reference's own FastxParser<DNA_SIMPLE>
// (include/goetia/parsing/readers.hh:150-219 over the vendored kseq.h) on
// FASTA/FASTQ files and prints what a caller of next() sees, so the C
// restatement in goetia_oracle.c and the committed FASTX fixtures are pinned
// to it.  Built by `make -C oracle ref-fastx`.
//
//   ref_fastx <min_length> <file>...
//
// Per file: "F <file>", one "S <sequence>" per read next() returns, then
// "P <n_parsed> K <n_skipped>" and, when next() threw InvalidRead, "E".
#include <cstdio>
#include <cstdlib>
#include <string>

#include "goetia/parsing/readers.hh"

int main(int argc, char** argv) {
    if (argc < 3) {
        std::fprintf(stderr, "usage: %s <min_length> <file>...\n", argv[0]);
        return 2;
    }
    const uint32_t min_length = (uint32_t)std::strtoul(argv[1], nullptr, 10);
    for (int a = 2; a < argc; ++a) {
        goetia::FastxParser<goetia::DNA_SIMPLE> parser(argv[a], false, min_length);
        std::printf("F %s\n", argv[a]);
        bool invalid = false;
        while (!parser.is_complete()) {
            try {
                auto rec = parser.next();
                if (rec) std::printf("S %s\n", rec->sequence.c_str());
            } catch (goetia::InvalidRead&) {
                invalid = true;
                break;
            }
        }
        std::printf("P %zu K %llu\n", parser.n_parsed(), (unsigned long long)parser.n_skipped());
        if (invalid) std::printf("E\n");
    }
    return 0;
}
