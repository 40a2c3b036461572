/* Stand-in for the CGAL kernel header: dcollid.cpp:23-25 only typedefs
 * Point_3 and Triangle_3 from it and never uses them. Test infrastructure only. */
#pragma once
namespace CGAL {
struct Exact_predicates_inexact_constructions_kernel {
    struct Point_3 {};
    struct Triangle_3 {};
};
}
