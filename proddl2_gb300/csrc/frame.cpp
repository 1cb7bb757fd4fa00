// Pre-scan frame set-up of a pair: MolStruct::moveIntoReferencePositions
// (include/PRODDL/docking_molstruct.hpp:199-252) and the grid size rule of
// FFTCorrelator::init (include/PRODDL/docking_fft.hpp:535-553).
//
//   1. spin the ligand about its centre of mass by the Euler angles
//      (s, 3.7877 s, -4.513432 s), s = startingSpin (randomizeLigandOrientation);
//   2. move both molecules into the receptor's box frame: rotate by the box
//      directions about the box centre (Box::moveToBoundCoordinates,
//      Geom/bounding.hpp:188-214);
//   3. move the ligand's diameter centre to the origin (Diameter,
//      bounding.hpp:27-76);
//   4. pad the receptor box by 2 h + ligand size / 2 + cutOffFft and pick the
//      FFT size per axis with findBestSize.
// Every transform is composed and applied with the reference's
// RotationTranslation algebra (Geom/transformation.hpp:135-345): products as
// ((m0 x0) + m1 x1) + m2 x2, no contraction.  The receptor box is axis-aligned
// (the reference's Box with fixed directions), supplied by the caller, or the
// minimum-volume box computed here as the reference's Box does with gdiam.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "fftdock.h"

namespace {

struct Rt {
    double r[9];
    double v[3];
};

void mat_vec(const double* m, const double* x, double* y) {
    for (int i = 0; i < 3; ++i) {
        double acc = m[3 * i] * x[0];
        acc = acc + m[3 * i + 1] * x[1];
        acc = acc + m[3 * i + 2] * x[2];
        y[i] = acc;
    }
}

void mat_mat(const double* a, const double* b, double* c) {
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double acc = a[3 * i] * b[j];
            acc = acc + a[3 * i + 1] * b[3 + j];
            acc = acc + a[3 * i + 2] * b[6 + j];
            c[3 * i + j] = acc;
        }
}

Rt identity() {
    Rt t;
    const double id[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    std::memcpy(t.r, id, sizeof(id));
    t.v[0] = t.v[1] = t.v[2] = 0.0;
    return t;
}

// a * b: apply b, then a
Rt compose(const Rt& a, const Rt& b) {
    Rt c;
    mat_mat(a.r, b.r, c.r);
    double p[3];
    mat_vec(a.r, b.v, p);
    for (int i = 0; i < 3; ++i) c.v[i] = p[i] + a.v[i];
    return c;
}

void apply(const Rt& t, double* p) {
    double q[3];
    mat_vec(t.r, p, q);
    for (int i = 0; i < 3; ++i) p[i] = q[i] + t.v[i];
}

// Eu_xyz::eulerAngToRotMatr (Geom/euler.hpp:38-52), radians
void euler_matrix(double a, double b, double g, double* m) {
    const double sa = std::sin(a), ca = std::cos(a), sb = std::sin(b), cb = std::cos(b), sg = std::sin(g),
                 cg = std::cos(g);
    const double r[9] = {cg * ca,
                         cg * sa,
                         -sg,
                         sb * sg * ca - cb * sa,
                         sb * sg * sa + cb * ca,
                         cg * sb,
                         cb * sg * ca + sb * sa,
                         cb * sg * sa - sb * ca,
                         cg * cb};
    std::memcpy(m, r, sizeof(r));
}

bool finite_all(const double* p, size_t n) {
    for (size_t i = 0; i < n; ++i)
        if (!std::isfinite(p[i])) return false;
    return true;
}

void pack(const Rt& t, double* out) {
    std::memcpy(out, t.r, 9 * sizeof(double));
    std::memcpy(out + 9, t.v, 3 * sizeof(double));
}

// ---------------------------------------------------------------------------
// Minimum-volume bounding box of the receptor: the approximation of Barequet
// and Har-Peled ("Efficiently approximating the minimum-volume bounding box of
// a point set in three dimensions", 2001) as the reference runs it through its
// gdiam library with grid 5 and every point (Geom::Bounding::Box,
// include/PRODDL/Geom/bounding.hpp:137-172):
//   1. a first box on the diameter direction, the diameter of the points
//      projected across it, and their cross product; the axis-parallel box
//      if that is smaller;
//   2. improvement: for each box direction in turn (10 times), project the
//      points onto the plane across it, take the minimum-area rectangle of
//      the projected convex hull (one edge of the hull lies on a side of the
//      optimal rectangle), and keep the new box if its volume is smaller;
//   3. search: every primitive integer combination (x, y, z) of the box's
//      directions with |x|, |y| <= grid and 0 <= z <= grid as the first
//      direction of a box built as in 2 and improved 10 times; the smallest
//      box wins and is improved once more.
// ---------------------------------------------------------------------------
double dot3(const double* a, const double* b) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }

void cross3(const double* a, const double* b, double* c) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}

bool normalize3(double* a) {
    const double l = std::sqrt(dot3(a, a));
    if (!(l > 0.0)) return false;
    for (int d = 0; d < 3; ++d) a[d] /= l;
    return true;
}

struct Box3 {
    double dir[3][3];  // rows
    double lo[3], hi[3];
    double vol() const { return ((hi[0] - lo[0]) * (hi[1] - lo[1])) * (hi[2] - lo[2]); }
};

Box3 bound_box(const std::vector<double>& pts, const double* a, const double* b, const double* c) {
    Box3 bx;
    const double* dirs[3] = {a, b, c};
    for (int k = 0; k < 3; ++k) {
        std::memcpy(bx.dir[k], dirs[k], 3 * sizeof(double));
        bx.lo[k] = INFINITY;
        bx.hi[k] = -INFINITY;
    }
    const size_t n = pts.size() / 3;
    for (size_t i = 0; i < n; ++i)
        for (int k = 0; k < 3; ++k) {
            const double v = dot3(&pts[3 * i], bx.dir[k]);
            bx.lo[k] = std::fmin(bx.lo[k], v);
            bx.hi[k] = std::fmax(bx.hi[k], v);
        }
    return bx;
}

// unit vectors u, v completing d (unit) to an orthonormal base
void complete_base(const double* d, double* u, double* v) {
    double ax[3] = {0.0, 0.0, 0.0};
    int m = 0;
    for (int k = 1; k < 3; ++k)
        if (std::fabs(d[k]) < std::fabs(d[m])) m = k;
    ax[m] = 1.0;
    cross3(d, ax, u);
    normalize3(u);
    cross3(d, u, v);
    normalize3(v);
}

double cross2(const double* o, const double* a, const double* b) {
    return (a[0] - o[0]) * (b[1] - o[1]) - (a[1] - o[1]) * (b[0] - o[0]);
}

// the box whose first direction is d and whose other two are the sides of
// the minimum-area rectangle around the points projected across d
Box3 proj_box(const std::vector<double>& pts, const double* d_in) {
    double d[3] = {d_in[0], d_in[1], d_in[2]};
    normalize3(d);
    double u[3], v[3];
    complete_base(d, u, v);
    const size_t n = pts.size() / 3;
    std::vector<double> q(2 * n);
    std::vector<int> idx(n);
    for (size_t i = 0; i < n; ++i) {
        q[2 * i] = dot3(&pts[3 * i], u);
        q[2 * i + 1] = dot3(&pts[3 * i], v);
        idx[i] = (int)i;
    }
    std::sort(idx.begin(), idx.end(), [&](int a, int b) {
        return q[2 * a] < q[2 * b] || (q[2 * a] == q[2 * b] && q[2 * a + 1] < q[2 * b + 1]);
    });
    // Andrew's monotone chain, counter-clockwise, collinear points dropped
    std::vector<int> h(2 * n + 1);
    size_t k = 0;
    for (size_t i = 0; i < n; ++i) {
        while (k >= 2 && cross2(&q[2 * h[k - 2]], &q[2 * h[k - 1]], &q[2 * idx[i]]) <= 0.0) --k;
        h[k++] = idx[i];
    }
    for (size_t i = n - 1, t = k + 1; i-- > 0;) {
        while (k >= t && cross2(&q[2 * h[k - 2]], &q[2 * h[k - 1]], &q[2 * idx[i]]) <= 0.0) --k;
        h[k++] = idx[i];
    }
    const size_t nh = k > 1 ? k - 1 : k;
    double e_best[2] = {1.0, 0.0};
    double best = INFINITY;
    for (size_t i = 0; i + 1 < k && nh >= 2; ++i) {
        double e[2] = {q[2 * h[i + 1]] - q[2 * h[i]], q[2 * h[i + 1] + 1] - q[2 * h[i] + 1]};
        const double l = std::sqrt(e[0] * e[0] + e[1] * e[1]);
        if (!(l > 0.0)) continue;
        e[0] /= l;
        e[1] /= l;
        double lo0 = INFINITY, hi0 = -INFINITY, lo1 = INFINITY, hi1 = -INFINITY;
        for (size_t j = 0; j < nh; ++j) {
            const double* p = &q[2 * h[j]];
            const double a = p[0] * e[0] + p[1] * e[1], b = p[1] * e[0] - p[0] * e[1];
            lo0 = std::fmin(lo0, a);
            hi0 = std::fmax(hi0, a);
            lo1 = std::fmin(lo1, b);
            hi1 = std::fmax(hi1, b);
        }
        const double area = (hi0 - lo0) * (hi1 - lo1);
        if (area < best) {
            best = area;
            e_best[0] = e[0];
            e_best[1] = e[1];
        }
    }
    double a3[3], b3[3];
    for (int c = 0; c < 3; ++c) {
        a3[c] = e_best[0] * u[c] + e_best[1] * v[c];
        b3[c] = -e_best[1] * u[c] + e_best[0] * v[c];
    }
    normalize3(a3);
    normalize3(b3);
    return bound_box(pts, d, a3, b3);
}

Box3 improve(const std::vector<double>& pts, Box3 bx, int times) {
    for (int i = 0; i < times; ++i) {
        const Box3 nb = proj_box(pts, bx.dir[i % 3]);
        if (nb.vol() < bx.vol()) bx = nb;
    }
    return bx;
}

int gcd_int(int a, int b) {
    a = std::abs(a);
    b = std::abs(b);
    while (b) {
        const int t = a % b;
        a = b;
        b = t;
    }
    return a;
}

// farthest pair (exact, the first pair in index order among equals) of the
// points, or of their projections across the unit vector `across`
void farthest(const std::vector<double>& pts, const double* across, int& bi, int& bj) {
    const size_t n = pts.size() / 3;
    double best = -1.0;
    bi = bj = 0;
    std::vector<double> p(pts);
    if (across)
        for (size_t i = 0; i < n; ++i) {
            const double t = dot3(&p[3 * i], across);
            for (int c = 0; c < 3; ++c) p[3 * i + c] -= t * across[c];
        }
    for (size_t i = 0; i < n; ++i)
        for (size_t j = i + 1; j < n; ++j) {
            const double dx = p[3 * j] - p[3 * i], dy = p[3 * j + 1] - p[3 * i + 1], dz = p[3 * j + 2] - p[3 * i + 2];
            const double d2 = (dx * dx + dy * dy) + dz * dz;
            if (d2 > best) {
                best = d2;
                bi = (int)i;
                bj = (int)j;
            }
        }
}

Box3 min_volume_box(const std::vector<double>& pts, int grid) {
    const double ex[3] = {1, 0, 0}, ey[3] = {0, 1, 0}, ez[3] = {0, 0, 1};
    const Box3 axes = bound_box(pts, ex, ey, ez);
    int i1, j1;
    farthest(pts, nullptr, i1, j1);
    double d1[3], d2[3], d3[3];
    for (int c = 0; c < 3; ++c) d1[c] = pts[3 * i1 + c] - pts[3 * j1 + c];
    if (!normalize3(d1)) return axes;  // all points coincide
    int i2, j2;
    farthest(pts, d1, i2, j2);
    for (int c = 0; c < 3; ++c) d2[c] = pts[3 * i2 + c] - pts[3 * j2 + c];
    const double pr = dot3(d1, d2);
    for (int c = 0; c < 3; ++c) d2[c] -= pr * d1[c];
    if (!normalize3(d2)) complete_base(d1, d2, d3);  // collinear points
    cross3(d1, d2, d3);
    normalize3(d3);
    Box3 bx = bound_box(pts, d1, d2, d3);
    if (axes.vol() < bx.vol()) bx = axes;
    bx = improve(pts, bx, 10);
    Box3 best = bx;
    for (int x = -grid; x <= grid; ++x)
        for (int y = -grid; y <= grid; ++y)
            for (int z = 0; z <= grid; ++z) {
                if ((x == 0 && y == 0 && z == 0) || gcd_int(gcd_int(x, y), z) > 1) continue;
                double dir[3];
                for (int c = 0; c < 3; ++c) dir[c] = (x * bx.dir[0][c] + y * bx.dir[1][c]) + z * bx.dir[2][c];
                if (!normalize3(dir)) continue;
                const Box3 nb = improve(pts, proj_box(pts, dir), 10);
                if (nb.vol() < best.vol()) best = nb;
            }
    return improve(pts, best, 10);
}

// direction rows and the corners (0,0,0) and (1,1,1) of a box, in the frame
// of its points
void box_corners(const Box3& bx, double* dirs, double* c0, double* c1) {
    for (int k = 0; k < 3; ++k) std::memcpy(dirs + 3 * k, bx.dir[k], 3 * sizeof(double));
    for (int c = 0; c < 3; ++c) {
        c0[c] = (bx.lo[0] * bx.dir[0][c] + bx.lo[1] * bx.dir[1][c]) + bx.lo[2] * bx.dir[2][c];
        c1[c] = (bx.hi[0] * bx.dir[0][c] + bx.hi[1] * bx.dir[1][c]) + bx.hi[2] * bx.dir[2][c];
    }
}

}  // namespace

extern "C" {

int fftdock_min_volume_box(int32_t n, const double* xyz, int32_t grid, double* dirs, double* corners) {
    if (n < 1 || !xyz || grid < 0 || grid > 16 || !dirs || !corners) return FFTDOCK_EINVAL;
    if (!finite_all(xyz, 3 * (size_t)n)) return FFTDOCK_EINVAL;
    const std::vector<double> pts(xyz, xyz + 3 * (size_t)n);
    const Box3 bx = min_volume_box(pts, grid);
    box_corners(bx, dirs, corners, corners + 3);
    return FFTDOCK_OK;
}

int fftdock_frame_setup(const fftdock_frame_setup_in* in, double* rec_out, double* lig_out, fftdock_frame* out) {
    if (!in || !out || in->n_rec < 1 || in->n_lig < 1 || !in->rec_xyz || !in->lig_xyz || !rec_out || !lig_out)
        return FFTDOCK_EINVAL;
    if (!(in->grid_step > 0.0) || !std::isfinite(in->cut_off_fft) || !std::isfinite(in->starting_spin))
        return FFTDOCK_EINVAL;
    if (in->box_mode != FFTDOCK_BOX_AXES && in->box_mode != FFTDOCK_BOX_GIVEN &&
        in->box_mode != FFTDOCK_BOX_MIN_VOLUME)
        return FFTDOCK_EINVAL;
    if (in->box_mode == FFTDOCK_BOX_GIVEN && (!in->box_dirs || !in->box_corners)) return FFTDOCK_EINVAL;
    const int nr = in->n_rec, nl = in->n_lig;
    if (!finite_all(in->rec_xyz, 3 * (size_t)nr) || !finite_all(in->lig_xyz, 3 * (size_t)nl)) return FFTDOCK_EINVAL;
    std::vector<double> rec(in->rec_xyz, in->rec_xyz + 3 * (size_t)nr);
    std::vector<double> lig(in->lig_xyz, in->lig_xyz + 3 * (size_t)nl);
    Rt tr_rec = identity(), tr_lig = identity();

    // 1. spin about the centre of mass: Translation(cm) * Rotation * Translation(-cm)
    double tot = 0.0;
    for (int i = 0; i < nl; ++i) {
        const double m = in->lig_mass ? in->lig_mass[i] : 1.0;
        if (!std::isfinite(m)) return FFTDOCK_EINVAL;
        tot = tot + m;
    }
    if (!(tot != 0.0)) return FFTDOCK_EINVAL;
    double cm[3] = {0.0, 0.0, 0.0};
    for (int i = 0; i < nl; ++i) {
        const double m = in->lig_mass ? in->lig_mass[i] : 1.0;
        for (int d = 0; d < 3; ++d) cm[d] = cm[d] + lig[3 * i + d] * m;
    }
    for (int d = 0; d < 3; ++d) cm[d] = cm[d] / tot;
    const double s = in->starting_spin;
    Rt spin;
    euler_matrix(s, s * 3.7877, s * -4.513432, spin.r);
    {
        const double neg[3] = {-1.0 * cm[0], -1.0 * cm[1], -1.0 * cm[2]};
        double p[3];
        mat_vec(spin.r, neg, p);
        for (int d = 0; d < 3; ++d) spin.v[d] = p[d] + cm[d];
    }
    for (int i = 0; i < nl; ++i) apply(spin, &lig[3 * i]);
    tr_lig = compose(spin, tr_lig);

    // 2. receptor box frame: Rotation(dirs) * Translation(-(c0 + (c1 - c0) / 2))
    double dirs[9], c0[3], c1[3];
    if (in->box_mode == FFTDOCK_BOX_GIVEN) {
        if (!finite_all(in->box_dirs, 9) || !finite_all(in->box_corners, 6)) return FFTDOCK_EINVAL;
        std::memcpy(dirs, in->box_dirs, sizeof(dirs));
        std::memcpy(c0, in->box_corners, sizeof(c0));
        std::memcpy(c1, in->box_corners + 3, sizeof(c1));
    } else if (in->box_mode == FFTDOCK_BOX_MIN_VOLUME) {
        const Box3 bx = min_volume_box(rec, 5);
        box_corners(bx, dirs, c0, c1);
    } else {
        const double id[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
        std::memcpy(dirs, id, sizeof(dirs));
        for (int d = 0; d < 3; ++d) c0[d] = c1[d] = rec[d];
        for (int i = 0; i < nr; ++i)
            for (int d = 0; d < 3; ++d) {
                c0[d] = std::fmin(c0[d], rec[3 * i + d]);
                c1[d] = std::fmax(c1[d], rec[3 * i + d]);
            }
    }
    Rt tb;
    std::memcpy(tb.r, dirs, sizeof(dirs));
    {
        double t[3];
        for (int d = 0; d < 3; ++d) t[d] = -(c0[d] + (c1[d] - c0[d]) / 2.0);
        mat_vec(dirs, t, tb.v);
    }
    double d0[3], d1[3];
    std::memcpy(d0, c0, sizeof(d0));
    std::memcpy(d1, c1, sizeof(d1));
    apply(tb, d0);
    apply(tb, d1);
    for (int i = 0; i < nr; ++i) apply(tb, &rec[3 * i]);
    for (int i = 0; i < nl; ++i) apply(tb, &lig[3 * i]);
    tr_rec = compose(tb, tr_rec);
    tr_lig = compose(tb, tr_lig);

    // 3. ligand diameter centre to the origin
    double p[3], q[3];
    if (in->lig_diam) {
        if (!finite_all(in->lig_diam, 6)) return FFTDOCK_EINVAL;
        std::memcpy(p, in->lig_diam, sizeof(p));
        std::memcpy(q, in->lig_diam + 3, sizeof(q));
    } else {
        double best = -1.0;
        int bi = 0, bj = 0;
        for (int i = 0; i < nl; ++i)
            for (int j = i + 1; j < nl; ++j) {
                const double dx = lig[3 * j] - lig[3 * i], dy = lig[3 * j + 1] - lig[3 * i + 1],
                             dz = lig[3 * j + 2] - lig[3 * i + 2];
                const double d2 = (dx * dx + dy * dy) + dz * dz;
                if (d2 > best) {
                    best = d2;
                    bi = i;
                    bj = j;
                }
            }
        std::memcpy(p, &lig[3 * bi], sizeof(p));
        std::memcpy(q, &lig[3 * bj], sizeof(q));
    }
    double tl[3];
    for (int d = 0; d < 3; ++d) tl[d] = -((q[d] + p[d]) / 2.0);
    for (int i = 0; i < nl; ++i)
        for (int d = 0; d < 3; ++d) lig[3 * i + d] = tl[d] + lig[3 * i + d];
    for (int d = 0; d < 3; ++d) tr_lig.v[d] = tr_lig.v[d] + tl[d];
    const double dd[3] = {q[0] - p[0], q[1] - p[1], q[2] - p[2]};
    const double lig_size = std::sqrt((dd[0] * dd[0] + dd[1] * dd[1]) + dd[2] * dd[2]);

    // 4. padded box and FFT sizes
    const double pad = (in->grid_step * 2.0 + lig_size / 2.0) + in->cut_off_fft;
    int32_t nmax = 0;
    for (int d = 0; d < 3; ++d) {
        const double lo = d0[d] - pad, hi = d1[d] + pad;
        out->min_box[d] = lo;
        out->min_box[3 + d] = hi;
        const double zero_h = lo - in->grid_step;
        const int start = (int)((hi - zero_h) / in->grid_step) - 1;
        int32_t n = 0;
        if (fftdock_find_best_size(start, &n) != FFTDOCK_OK) return FFTDOCK_EINVAL;
        out->fft_size[d] = n;
        if (n > nmax) nmax = n;
    }
    out->grid_n = 0;
    for (int n = nmax; n <= 1024; ++n)
        if (fftdock_supported_grid(n)) {
            out->grid_n = n;
            break;
        }
    out->lig_size = lig_size;
    pack(tr_rec, out->rec_frame);
    pack(tr_lig, out->lig_frame);
    std::memcpy(rec_out, rec.data(), rec.size() * sizeof(double));
    std::memcpy(lig_out, lig.data(), lig.size() * sizeof(double));
    return FFTDOCK_OK;
}

}  // extern "C"
