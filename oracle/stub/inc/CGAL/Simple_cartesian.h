/* Empty stand-in for CGAL/Simple_cartesian.h: the collision sources include it but call
 * nothing from it (the CGAL box-intersection path is commented out,
 * dcollid.cpp:246-252, 392-400, 444-451). Test infrastructure only. */
#pragma once
