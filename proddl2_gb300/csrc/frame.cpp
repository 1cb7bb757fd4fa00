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
// (the reference's Box with fixed directions) or supplied by the caller (the
// reference's own minimum-volume box, which it takes from the gdiam library).
#include <cmath>
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

}  // namespace

extern "C" {

int fftdock_frame_setup(const fftdock_frame_setup_in* in, double* rec_out, double* lig_out, fftdock_frame* out) {
    if (!in || !out || in->n_rec < 1 || in->n_lig < 1 || !in->rec_xyz || !in->lig_xyz || !rec_out || !lig_out)
        return FFTDOCK_EINVAL;
    if (!(in->grid_step > 0.0) || !std::isfinite(in->cut_off_fft) || !std::isfinite(in->starting_spin))
        return FFTDOCK_EINVAL;
    if (in->box_mode != FFTDOCK_BOX_AXES && in->box_mode != FFTDOCK_BOX_GIVEN) return FFTDOCK_EINVAL;
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
