// A report that records every pair it is called with (a client-defined
// report type: pbig_check must inline this operator(), not the counting one).
#ifndef __REPORT_H
#define __REPORT_H
#include <vector>
#include "rect.h"
struct report {
public:
    report();
    void operator()(unsigned int a, unsigned int b) { pairs.push_back(a); pairs.push_back(b); }
    void print();
    std::vector<unsigned int> pairs;
};
#endif
