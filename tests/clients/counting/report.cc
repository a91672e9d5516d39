#include <stdio.h>
#include "report.h"
report::report() : sum(0) {}
void report::print() { printf("Number of pairs = %d\n", sum); }
void report::found(const RectInfo* a, const RectInfo* b) { sum++; }
