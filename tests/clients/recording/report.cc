#include <stdio.h>
#include <stdlib.h>
#include "report.h"
report::report() {}
// writes the pairs as binary uint32 (a, b) records to $PBIG_PAIRS_OUT
void report::print() {
    const char* path = getenv("PBIG_PAIRS_OUT");
    printf("Number of pairs = %zu\n", pairs.size() / 2);
    if (!path) return;
    FILE* f = fopen(path, "wb");
    if (!f) return;
    fwrite(pairs.data(), 4, pairs.size(), f);
    fclose(f);
}
