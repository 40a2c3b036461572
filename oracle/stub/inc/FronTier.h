/*
 * Minimal stand-in for the FronTier front-tracking library, written for this
 * project so that the collision sources of antdvid/Collision (AABB.cpp,
 * dcollid.cpp, dcollid3d.cpp) compile unmodified as a CPU test oracle.
 *
 * TEST INFRASTRUCTURE ONLY: nothing in the shipped library includes this.
 *
 * FronTier itself is not vendored by the reference (Makefile:17-22 link
 * -lFronTier from ../lib) and its version is unknown, so the vector macros and
 * constants below pin an assumption:
 *   Dot3d      left-to-right a0*b0 + a1*b1 + a2*b2
 *   Mag3d      sqrt(Dot3d(a,a))
 *   Cross3d    standard right-handed cross product
 *   sqr        x*x
 *   distance_between_positions   sqrt of the left-to-right sum of squares
 *   MACH_EPS   DBL_EPSILON
 *   HUGE       1.0e38 when <math.h> does not provide it; the reference only
 *              uses it as a min/max identity (dcollid.cpp:863-930), far
 *              beyond any coordinate, so its exact value never matters.
 */
#ifndef ORACLE_STUB_FRONTIER_H
#define ORACLE_STUB_FRONTIER_H

#include <cmath>
#include <cfloat>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fenv.h>
#include <vector>
#include <map>
#include <algorithm>
#include <iostream>

#define YES true
#define NO false
#define ERROR (-1)
#define MACH_EPS DBL_EPSILON
#ifndef HUGE
#define HUGE 1.0e38
#endif

typedef void* POINTER;
typedef struct _Front Front;   /* only named in collid.h prototypes */

enum { STRING_HSBDRY = 1, OTHER_HSBDRY = 0 };

struct HYPER_SURF {
    int body_index;
    double com[3];
    double comv[3];
    double mass;
};

struct POINT {
    double _coords[3];
    POINTER _left_state;
    POINTER _right_state;
    int _sorted;
    long global_index;
    double vel[3];
    HYPER_SURF* hs;
    int indx;
};

struct SURFACE;

struct TRI {
    POINT* __pts[3];
    TRI* next;
    SURFACE* surf;
    double side_length0[3];
};

struct SURFACE {
    TRI* first;          /* first tri of the surface */
    TRI* tail_sentinel;  /* one past the last tri: the list terminator */
    int bdry;            /* is_bdry() */
    HYPER_SURF hs;
};

struct BOND {
    POINT* start;
    POINT* end;
    BOND* next;
    double length0;
};

struct CURVE {
    BOND* first;
    BOND* last;
    int hsb_type;        /* hsbdry_type() */
};

struct RECT_GRID {
    double L[3];
    double U[3];
};

struct INTFC_TABLE {
    RECT_GRID rect_grid;
};

struct INTERFACE {
    SURFACE** surfaces;  /* NULL-terminated */
    CURVE** curves;      /* NULL-terminated */
    INTFC_TABLE* table;
};

#define Coords(p) ((p)->_coords)
#define left_state(p) ((p)->_left_state)
#define right_state(p) ((p)->_right_state)
#define sorted(p) ((p)->_sorted)
#define Point_of_tri(tri) ((tri)->__pts)
#define first_tri(s) ((s)->first)
#define at_end_of_tri_list(tri, s) ((tri) == (s)->tail_sentinel)
#define surf_tri_loop(s, tri) \
    for ((tri) = first_tri(s); !at_end_of_tri_list(tri, s); (tri) = (tri)->next)
#define intfc_surface_loop(intfc, s) \
    for ((s) = (intfc)->surfaces; (s) && *(s); ++(s))
#define intfc_curve_loop(intfc, c) \
    for ((c) = (intfc)->curves; (c) && *(c); ++(c))
#define curve_bond_loop(c, b) for ((b) = (c)->first; (b) != NULL; (b) = (b)->next)
#define is_bdry(s) ((s)->bdry)
#define hsbdry_type(c) ((c)->hsb_type)
#define body_index(hs) ((hs)->body_index)
#define center_of_mass(hs) ((hs)->com)
#define center_of_mass_velo(hs) ((hs)->comv)
#define total_mass(hs) ((hs)->mass)

#define sqr(x) ((x) * (x))
#define Dot3d(a, b) ((a)[0] * (b)[0] + (a)[1] * (b)[1] + (a)[2] * (b)[2])
#define Mag3d(a) sqrt(Dot3d(a, a))
#define Cross3d(B, C, ANS)                           \
    do {                                             \
        (ANS)[0] = (B)[1] * (C)[2] - (B)[2] * (C)[1]; \
        (ANS)[1] = (B)[2] * (C)[0] - (B)[0] * (C)[2]; \
        (ANS)[2] = (B)[0] * (C)[1] - (B)[1] * (C)[0]; \
    } while (0)

inline double distance_between_positions(const double* p, const double* q, int dim) {
    double s = 0.0;
    for (int i = 0; i < dim; ++i) s += sqr(p[i] - q[i]);
    return sqrt(s);
}

/* Hooks supplied by the harness (oracle/ref_harness.cpp). */
bool debugging(const char*);
void clean_up(int);
void start_clock(const char*);
void stop_clock(const char*);
double cpu_seconds();
bool create_directory(const char*, bool);

#endif
