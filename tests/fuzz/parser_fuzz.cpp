// parser_fuzz.cpp — test infrastructure: mutates real streams (bit flips,
// overwritten runs, truncation, dropped and duplicated pieces, any
// chunking) and runs the host front end on each, to be built with
// AddressSanitizer and UndefinedBehaviorSanitizer by tests/test_parser.py.
// Every run must end with pictures or an error code, with no sanitizer
// report.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <vector>
#include "h264r_parser.h"
static std::vector<uint8_t> load(const char *p) { FILE *f = fopen(p, "rb"); std::vector<uint8_t> d(1 << 22); d.resize(fread(d.data(), 1, d.size(), f)); fclose(f); return d; }
int main(int argc, char **argv) {
    // usage: parser_fuzz <runs per stream> <stream.h264>...
    const int runs = atoi(argv[1]);
    std::mt19937 rng(12345);
    int errors = 0, pics = 0;
    for (int a = 2; a < argc; a++) {
        std::vector<uint8_t> base = load(argv[a]);
        std::vector<size_t> starts;
        for (size_t i = 0; i + 3 < base.size(); i++) if (base[i] == 0 && base[i+1] == 0 && base[i+2] == 1) starts.push_back(i);
        for (int t = 0; t < runs; t++) {
            std::vector<uint8_t> b = base;
            int kind = t % 5;
            if (kind == 0) { int n = 1 + rng() % 16; for (int k = 0; k < n; k++) b[rng() % b.size()] ^= 1u << (rng() % 8); }
            else if (kind == 1) { size_t i = rng() % (b.size() - 256); for (int k = 0; k < 256; k++) b[i + k] = rng(); }
            else if (kind == 2) { b.resize(rng() % b.size()); }
            else if (kind == 3) { size_t k = 1 + rng() % (starts.size() - 2); b.erase(b.begin() + starts[k], b.begin() + starts[k + 1]); }
            else { size_t i = rng() % b.size(), s0 = rng() % b.size(), n = 1 + rng() % 512; std::vector<uint8_t> piece(b.begin() + s0, b.begin() + std::min(b.size(), s0 + n)); b.insert(b.begin() + i, piece.begin(), piece.end()); }
            h264r_parser *p; h264r_parser_create(&p);
            size_t chunk = (t & 1) ? 997 : b.size();
            int rc = 0;
            for (size_t o = 0; o < b.size() && rc == 0; o += chunk) rc = h264r_parser_feed(p, b.data() + o, std::min(chunk, b.size() - o));
            if (rc == 0) rc = h264r_parser_end(p);
            h264r_parsed out;
            int r;
            while ((r = h264r_parser_next(p, &out)) == 1) { pics++; }
            if (rc || r < 0) errors++;
            h264r_parser_destroy(p);
        }
    }
    printf("fuzz done: %d runs with errors, %d pictures\n", errors, pics);
}
