// Project-written stand-in for CGAL::Triangulation_2 (TEST INFRASTRUCTURE ONLY): the types and
// members the reference's L-infinity retriangulation names, so integration.cpp compiles. That rule
// is outside the checked assembly path; inserting points aborts with a message.
#pragma once
#include <cstdio>
#include <cstdlib>
namespace CGAL {
template <typename K>
class Triangulation_2 {
  public:
    typedef typename K::Point_2 Point;
    struct Vertex {
        Point p;
        const Point &point() const { return p; }
    };
    struct Face {
        Vertex v[3];
        const Vertex *vertex(int k) const { return &v[k]; }
    };
    struct Finite_faces_iterator {
        const Face *f = nullptr;
        const Face *operator->() const { return f; }
        Finite_faces_iterator &operator++() { ++f; return *this; }
        bool operator!=(const Finite_faces_iterator &o) const { return f != o.f; }
        bool operator==(const Finite_faces_iterator &o) const { return f == o.f; }
    };
    template <typename It>
    void insert(It, It) {
        std::fprintf(stderr, "refshim: the L-infinity ball rules need CGAL, which this build does not have\n");
        std::abort();
    }
    Finite_faces_iterator finite_faces_begin() const { return Finite_faces_iterator(); }
    Finite_faces_iterator finite_faces_end() const { return Finite_faces_iterator(); }
};
}  // namespace CGAL
