/*
 * report.h — the pair-callback object of the PBIG API. A client normally
 * supplies its own report.h; this one has the shape of package/report.h of
 * awatch/pbig (a counter) and is what the prebuilt libpbig.a is compiled
 * against. pbig_check inlines report::operator() from whichever report.h is
 * first on the include path when legacy_pbig.cc is compiled.
 */
#ifndef __REPORT_H
#define __REPORT_H

#include "rect.h"

struct report {
public:
    report();
    void operator()(unsigned int a, unsigned int b) { sum++; }
    void found(const RectInfo* a, const RectInfo* b);
    void print();
    void reset() { sum = 0; }

private:
    int sum;
};

#endif
