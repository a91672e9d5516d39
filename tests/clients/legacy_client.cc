// A client of the pbig.h API in the style of the reference's example program
// (package/main.cc of awatch/pbig): pbig_init once, pbig_check per step with
// a report object, pbig_finalize. It reads RectInfo records from a binary
// file so that a test can hand it any scene, and prints the report.
//
//   legacy_client <boxes.bin> <num> <range> <steps> [cs]
#include <stdio.h>
#include <stdlib.h>
#include <sys/time.h>

#include "pbig.h"
#include "rect.h"
#include "report.h"

int main(int argc, char** argv) {
    if (argc < 5) {
        fprintf(stderr, "usage: %s boxes.bin num range steps [cs]\n", argv[0]);
        return 2;
    }
    unsigned num = (unsigned)strtoul(argv[2], 0, 10);
    unsigned range = (unsigned)strtoul(argv[3], 0, 10);
    int steps = atoi(argv[4]);
    unsigned cs = argc > 5 ? (unsigned)strtoul(argv[5], 0, 10) : 0;
    RectInfo* input = (RectInfo*)malloc(sizeof(RectInfo) * (num ? num : 1));
    FILE* f = fopen(argv[1], "rb");
    if (!f || fread(input, sizeof(RectInfo), num, f) != num) {
        fprintf(stderr, "cannot read %u boxes from %s\n", num, argv[1]);
        return 2;
    }
    fclose(f);
    pbig_init(num, range, cs, 0, 0);
    for (int s = 0; s < steps; s++) {
        report r;
        struct timeval b, e;
        gettimeofday(&b, 0);
        pbig_check(input, &r);
        gettimeofday(&e, 0);
        r.print();
        printf("step%d,%ld us\n", s, 1000000L * (e.tv_sec - b.tv_sec) + e.tv_usec - b.tv_usec);
    }
    pbig_finalize();
    free(input);
    return 0;
}
