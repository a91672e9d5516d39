/*
 * rect.h — box record of the PBIG API (layout of src/pbig/rect.h:4-18 and
 * package/rect.h:1-18 in awatch/pbig; kept identical so existing callers and
 * their data work unchanged). DIMS selects 2-D or 3-D records; the package
 * build of the reference is 3-D only, which is the default here.
 */
#ifndef __RECT_H_
#define __RECT_H_

#ifndef DIMS
#define DIMS 3
#endif

typedef unsigned int CType;

typedef struct CoordInfo {
    CType xmin, xmax;
    CType ymin, ymax;
#if DIMS == 3
    CType zmin, zmax;
#endif
} CoordInfo;

typedef struct RectInfo {
    CoordInfo coordinate;
    unsigned int rid; /* must equal the record's index in the input array */
} RectInfo;

#endif
