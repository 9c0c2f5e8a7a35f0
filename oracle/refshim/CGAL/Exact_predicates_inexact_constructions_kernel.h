// Project-written stand-in for the CGAL kernel type the reference's integration.h names (TEST
// INFRASTRUCTURE ONLY). Only the L-infinity ball rules use CGAL; they are outside the assembly
// path that the reference build checks, and the stand-in triangulation below aborts if one runs.
#pragma once
namespace CGAL {
struct Exact_predicates_inexact_constructions_kernel {
    struct Point_2 {
        double px = 0, py = 0;
        Point_2() {}
        Point_2(double x, double y) : px(x), py(y) {}
        double x() const { return px; }
        double y() const { return py; }
    };
};
}  // namespace CGAL
