// Gather of per-rotation scan records into the global ranked pose list, and
// the pose file the reference's export step reads.
//
// fftdock_gather_*  : Foreman::run (include/PRODDL/docking_app.hpp:174-220)
//                     over RotFftScanIO_Collector (docking_io_bin.hpp:81-116)
// fftdock_write_rigid: Foreman::writeResults (docking_app.hpp:269-281) with
//                     MolStruct::toOriginalFrame (docking_molstruct.hpp:31-51)
//                     and IORigid::writeCoords (IO/rigid.hpp:115-176)
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <string>
#include <utility>
#include <vector>

#include "fftdock.h"

namespace {

struct Rt {
    double r[9];
    double v[3];
};

// blitz_ext::product order: ((m0 x0) + m1 x1) + m2 x2
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

// a * b: apply b, then a
Rt compose(const Rt& a, const Rt& b) {
    Rt c;
    mat_mat(a.r, b.r, c.r);
    double p[3];
    mat_vec(a.r, b.v, p);
    for (int i = 0; i < 3; ++i) c.v[i] = p[i] + a.v[i];
    return c;
}

// RotationTranslation::inverse: (R^T, R^T (0 - v))
Rt inverse(const Rt& a) {
    Rt b;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) b.r[3 * i + j] = a.r[3 * j + i];
    const double nv[3] = {0.0 - a.v[0], 0.0 - a.v[1], 0.0 - a.v[2]};
    mat_vec(b.r, nv, b.v);
    return b;
}

// Eu_xyz::rotMatrToEulerAng (Geom/euler.hpp:58-102)
void euler(const double* m, double* out) {
    const double half_pi = 4.0 * std::atan(1.0) / 2.0;
    double a0, a1, a2;
    if (m[2] < 1.0) {
        if (m[2] > -1.0) {
            a0 = std::atan2(-m[5], m[8]);
            a1 = std::asin(m[2]);
            a2 = std::atan2(-m[1], m[0]);
        } else {
            a0 = -std::atan2(m[3], m[4]);
            a1 = -half_pi;
            a2 = 0.0;
        }
    } else {
        a0 = std::atan2(m[3], m[4]);
        a1 = half_pi;
        a2 = 0.0;
    }
    out[0] = -a2;
    out[1] = -a0;
    out[2] = -a1;
}

Rt frame_or_identity(const double* f) {
    Rt t;
    if (f) {
        std::memcpy(t.r, f, 9 * sizeof(double));
        std::memcpy(t.v, f + 9, 3 * sizeof(double));
    } else {
        const double id[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
        std::memcpy(t.r, id, sizeof(id));
        t.v[0] = t.v[1] = t.v[2] = 0.0;
    }
    return t;
}

// BoundPriorityQueue<RotTranValue> (Common/queue.hpp:221-251) with the value
// limit 1e16 of Foreman::init; ties keep arrival order
struct Entry {
    double value;
    int64_t seq;
    fftdock_pose pose;
};
bool worse(const Entry& a, const Entry& b) { return a.value > b.value || (a.value == b.value && a.seq > b.seq); }

struct PoseQueue {
    std::vector<Entry> heap;  // max-heap on (value, seq)
    size_t limit;
    int64_t seq = 0;
    explicit PoseQueue(size_t l) : limit(l) {}
    void sift_up(size_t i) {
        while (i > 0) {
            size_t p = (i - 1) / 2;
            if (!worse(heap[i], heap[p])) break;
            std::swap(heap[i], heap[p]);
            i = p;
        }
    }
    void sift_down(size_t i) {
        for (;;) {
            size_t l = 2 * i + 1, r = l + 1, m = i;
            if (l < heap.size() && worse(heap[l], heap[m])) m = l;
            if (r < heap.size() && worse(heap[r], heap[m])) m = r;
            if (m == i) return;
            std::swap(heap[i], heap[m]);
            i = m;
        }
    }
    void push(double value, const fftdock_pose& p) {
        Entry e{value, seq++, p};
        if (!(value < 1e16)) return;
        if (heap.size() >= limit) {
            if (worse(heap[0], e)) {
                heap[0] = e;
                sift_down(0);
            }
            return;
        }
        heap.push_back(e);
        sift_up(heap.size() - 1);
    }
};

// RotFftScanIO_Bin::read_record (docking_io_bin.hpp:34-53); returns 1 on a
// record, 0 at the end of the file, -1 on a signature mismatch
int read_record(std::FILE* f, double* rot, std::vector<double>& tv) {
    int32_t sig = 0;
    if (std::fread(&sig, sizeof(sig), 1, f) != 1) return 0;
    if (sig != 2014011401) return -1;
    if (std::fread(rot, sizeof(double), 9, f) != 9) return 0;
    uint64_t n = 0;
    if (std::fread(&n, sizeof(n), 1, f) != 1) return 0;
    if (n > (1ull << 32)) return -1;
    tv.resize((size_t)n * 4);
    if (n && std::fread(tv.data(), sizeof(double), (size_t)n * 4, f) != (size_t)n * 4) return 0;
    return 1;
}

int gather_files(const std::vector<std::string>& paths, int32_t max_matches, fftdock_pose* out, int32_t* n_out) {
    if (max_matches < 1 || !out || !n_out) return FFTDOCK_EINVAL;
    PoseQueue q((size_t)max_matches);
    std::vector<double> tv;
    double rot[9];
    for (const std::string& path : paths) {
        std::FILE* f = std::fopen(path.c_str(), "rb");
        if (!f) return FFTDOCK_EIO;
        for (;;) {
            const int rc = read_record(f, rot, tv);
            if (rc < 0) {
                std::fclose(f);
                return FFTDOCK_EIO;
            }
            if (rc == 0) break;
            const size_t n = tv.size() / 4;
            for (size_t i = 0; i < n; ++i) {
                // Translation(t) * Rotation(rot) = (rot, t)
                fftdock_pose p;
                p.value = tv[4 * i + 3];
                std::memcpy(p.rot, rot, sizeof(rot));
                p.t[0] = tv[4 * i];
                p.t[1] = tv[4 * i + 1];
                p.t[2] = tv[4 * i + 2];
                q.push(p.value, p);
            }
        }
        std::fclose(f);
    }
    std::vector<Entry> all(q.heap.begin(), q.heap.end());
    std::sort(all.begin(), all.end(), [](const Entry& a, const Entry& b) { return worse(b, a); });
    for (size_t i = 0; i < all.size(); ++i) out[i] = all[i].pose;
    *n_out = (int32_t)all.size();
    return FFTDOCK_OK;
}

}  // namespace

extern "C" {

int fftdock_gather_records(const char* const* paths, int32_t n_paths, int32_t max_matches, fftdock_pose* out,
                           int32_t* n_out) {
    if (n_paths < 0 || (n_paths > 0 && !paths)) return FFTDOCK_EINVAL;
    std::vector<std::string> p;
    for (int i = 0; i < n_paths; ++i) {
        if (!paths[i]) return FFTDOCK_EINVAL;
        p.emplace_back(paths[i]);
    }
    return gather_files(p, max_matches, out, n_out);
}

int fftdock_gather_list(const char* list_path, int32_t max_matches, fftdock_pose* out, int32_t* n_out) {
    if (!list_path) return FFTDOCK_EINVAL;
    std::ifstream in(list_path);
    if (!in.good()) return FFTDOCK_EIO;
    std::vector<std::string> p;
    std::string line;
    while (std::getline(in, line))
        if (!line.empty()) p.push_back(line);
    return gather_files(p, max_matches, out, n_out);
}

int fftdock_write_rigid(const char* path, const fftdock_pose* poses, int32_t n, const double* rec_frame,
                        const double* lig_frame, int32_t text) {
    if (!path || n < 0 || (n > 0 && !poses)) return FFTDOCK_EINVAL;
    const Rt inv_r = inverse(frame_or_identity(rec_frame));
    const Rt tl = frame_or_identity(lig_frame);
    std::vector<float> rec((size_t)n * 7);
    for (int i = 0; i < n; ++i) {
        Rt p;
        std::memcpy(p.r, poses[i].rot, sizeof(p.r));
        std::memcpy(p.v, poses[i].t, sizeof(p.v));
        const Rt o = compose(compose(inv_r, p), tl);
        double ang[3];
        euler(o.r, ang);
        float* r = &rec[(size_t)i * 7];
        r[0] = (float)poses[i].value;
        for (int d = 0; d < 3; ++d) {
            r[1 + d] = (float)ang[d];
            r[4 + d] = (float)o.v[d];
        }
    }
    if (!text) {
        std::FILE* f = std::fopen(path, "wb");
        if (!f) return FFTDOCK_EIO;
        const int32_t sig = 2005052501, nn = n;
        bool ok = std::fwrite(&sig, sizeof(sig), 1, f) == 1 && std::fwrite(&nn, sizeof(nn), 1, f) == 1;
        ok = ok && (n == 0 || std::fwrite(rec.data(), sizeof(float) * 7, (size_t)n, f) == (size_t)n);
        if (std::fclose(f) != 0) ok = false;
        return ok ? FFTDOCK_OK : FFTDOCK_EIO;
    }
    std::FILE* f = std::fopen(path, "w");
    if (!f) return FFTDOCK_EIO;
    bool ok = std::fprintf(f, "%d\n", n) > 0;
    for (int i = 0; i < n && ok; ++i) {
        const float* r = &rec[(size_t)i * 7];
        ok = std::fprintf(f, "%#.10g\t%#.10g\t%#.10g\t%#.10g\t%#.10g\t%#.10g\t%#.10g\n", r[0], r[1], r[2], r[3], r[4],
                          r[5], r[6]) > 0;
    }
    if (std::fclose(f) != 0) ok = false;
    return ok ? FFTDOCK_OK : FFTDOCK_EIO;
}

}  // extern "C"
