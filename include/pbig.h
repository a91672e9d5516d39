/*
 * pbig.h — the PBIG library API (same declarations as src/pbig/pbig.h:9-11
 * and package/pbig.h:9-11 of awatch/pbig, so clients compile and link
 * unchanged against this engine).
 *
 *   pbig_init(num, range, cs, deviceID, hasProfSteps)
 *       num: boxes passed to every later pbig_check; range: every coordinate
 *       is < range; cs: 0 = automatic cell size (a power of two selects that
 *       cell size); deviceID: CUDA device; hasProfSteps: ignored.
 *   pbig_check(input, r)
 *       calls (*r)(a, b) once for every unordered pair of overlapping boxes
 *       (closed intervals on every axis), on the calling thread, before
 *       returning. a and b are the boxes' rid values.
 *   pbig_finalize()
 *       releases the engine (other CUDA users of the process are unaffected).
 */
#ifndef __PBIG_H_
#define __PBIG_H_

using namespace std;
#include <set>
#include <vector>

struct report;
void pbig_init(unsigned int, unsigned int, unsigned int, unsigned int, unsigned int);
void pbig_check(struct RectInfo*, struct report*);
void pbig_finalize();

#endif
