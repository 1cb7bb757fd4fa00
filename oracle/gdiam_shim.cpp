// Test-only C entry points to the reference's gdiam wrappers
// (src/PRODDL/Geom/gdiam_simple.cpp), compiled together with the reference's
// own sources into oracle/_ref by oracle/build_ref.py.  Used to pin the frame
// set-up's diameter and box handling against the reference itself.
#include "PRODDL/Geom/gdiam_simple.hpp"

extern "C" {

// gdiam_approx_diam_pair with eps; out = end point p, then q
void ref_diam_pair(const double* pts, int n, double eps, double* out) {
    PRODDL::Geom::Gdiam::simp_approx_diam_pair(pts, n, out, out + 3, eps);
}

// gdiam_approx_mvbb_grid_sample as Geom::Bounding::Box calls it; corners =
// vertex (0,0,0) then vertex (1,1,1); dirs = the 3 direction rows
void ref_mvbb(const double* pts, int n, int grid_n, int sample_n, double* corners, double* dirs) {
    PRODDL::Geom::Gdiam::simp_approx_mvbb_grid_sample(pts, n, corners, corners + 3, dirs, grid_n, sample_n);
}

}
