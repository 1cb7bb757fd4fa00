// fftdock-scan: command-line front end with the tasks and option names of the
// reference's proddl-dock-fft (src/PRODDL/docking_main.cpp:55-66,101-136).
//
//   fftdock-scan --task rot-scan --options scan.json --molforce-params pair.txt
//                --fft-rot-grid-start S --fft-rot-grid-end E --fft-rot-scan-res out.dat
//   fftdock-scan --task gather --options scan.json --fft-rot-scan-list list.tab
//                --fft-res out.rigid [--molforce-params pair.txt]
//
// rot-scan writes one RotFftScanIO_Bin record per rotation of
// [start, end) of the options' "anglesFile" (docking_app.hpp:326-513);
// gather merges the listed record files into the maxNRigidMatches best poses
// and writes them as IORigid (docking_app.hpp:117-313).
//
// Options (JSON; keys are looked up anywhere in the file, the reference keeps
// them in its "scan" block): gridStep, maxNTrans, maxNTransInp, maxValCorr,
// cutOffFft, anglesFile, maxNRigidMatches, doClusterTranslations,
// clusterRadiusTrans, plus gridN (grid edge; default: the reference's size
// rule over the padded receptor box), termSet ("shape" or "shape_ace"),
// rotBatch, clusterOrder ("reference" or "best_first"), potentialName
// ("ljComp" / "ljAvg": the reference's LJ potentials, with cutOffFft and
// ljMix).
//
// The reference reads atoms from an HDF5 molforce file built with IMP; this
// front end reads a text pair file instead:
//   receptor <n>          then n lines "x y z type"
//   ligand <m>            then m lines "x y z type"
//   ace <T>               then T lines of T numbers (desolvation matrix)
//   receptor_lj <n>       then n lines "sigma eps alpha" (LJ potentials)
//   ligand_lj <m>         then m lines "sigma eps"
//   receptor_frame / ligand_frame  12 numbers each (optional; row-major
//                         rotation then vector, mapping original to scan frame)
// Lines starting with '#' are comments.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "fftdock.h"

namespace {

[[noreturn]] void die(const std::string& msg, int code = 1) {
    std::fprintf(stderr, "fftdock-scan: %s\n", msg.c_str());
    std::exit(code);
}

// flat scalar map of a JSON document: "key": number|string|bool
std::map<std::string, std::string> read_json_scalars(const std::string& path) {
    std::ifstream in(path);
    if (!in.good()) die("cannot open options file " + path);
    std::stringstream ss;
    ss << in.rdbuf();
    const std::string s = ss.str();
    std::map<std::string, std::string> out;
    size_t i = 0;
    while ((i = s.find('"', i)) != std::string::npos) {
        const size_t j = s.find('"', i + 1);
        if (j == std::string::npos) break;
        const std::string key = s.substr(i + 1, j - i - 1);
        size_t k = j + 1;
        while (k < s.size() && std::isspace((unsigned char)s[k])) ++k;
        if (k < s.size() && s[k] == ':') {
            ++k;
            while (k < s.size() && std::isspace((unsigned char)s[k])) ++k;
            if (k < s.size() && s[k] == '"') {
                const size_t e = s.find('"', k + 1);
                if (e == std::string::npos) break;
                out[key] = s.substr(k + 1, e - k - 1);
                i = e + 1;
                continue;
            }
            if (k < s.size() && s[k] != '{' && s[k] != '[') {
                size_t e = k;
                while (e < s.size() && s[e] != ',' && s[e] != '}' && s[e] != '\n') ++e;
                std::string v = s.substr(k, e - k);
                while (!v.empty() && std::isspace((unsigned char)v.back())) v.pop_back();
                out[key] = v;
                i = e;
                continue;
            }
        }
        i = j + 1;
    }
    return out;
}

double num(const std::map<std::string, std::string>& o, const char* key, double dflt) {
    auto it = o.find(key);
    if (it == o.end()) return dflt;
    if (it->second == "Infinity" || it->second == "inf") return INFINITY;
    if (it->second == "true") return 1.0;
    if (it->second == "false") return 0.0;
    char* end = nullptr;
    const double v = std::strtod(it->second.c_str(), &end);
    if (end == it->second.c_str()) die(std::string("option ") + key + " is not a number");
    return v;
}

struct Pair {
    std::vector<double> rec_xyz, lig_xyz, ace;
    std::vector<double> rec_lj, lig_lj;  // per atom (sigma, eps, alpha) / (sigma, eps)
    std::vector<int32_t> rec_type, lig_type;
    int n_types = 0;
    bool has_rec_frame = false, has_lig_frame = false;
    double rec_frame[12], lig_frame[12];
};

Pair read_pair(const std::string& path) {
    std::ifstream in(path);
    if (!in.good()) die("cannot open pair file " + path);
    Pair p;
    std::string word;
    auto atoms = [&](int n, std::vector<double>& xyz, std::vector<int32_t>& type) {
        for (int i = 0; i < n; ++i) {
            double x, y, z;
            int t;
            if (!(in >> x >> y >> z >> t)) die("truncated atom list in " + path);
            xyz.insert(xyz.end(), {x, y, z});
            type.push_back(t);
        }
    };
    while (in >> word) {
        if (word[0] == '#') {
            std::string rest;
            std::getline(in, rest);
            continue;
        }
        if (word == "receptor" || word == "ligand") {
            int n;
            if (!(in >> n) || n < 0) die("bad atom count in " + path);
            if (word == "receptor") atoms(n, p.rec_xyz, p.rec_type);
            else atoms(n, p.lig_xyz, p.lig_type);
        } else if (word == "receptor_lj" || word == "ligand_lj") {
            int n;
            if (!(in >> n) || n < 0) die("bad atom count in " + path);
            const int per = word == "receptor_lj" ? 3 : 2;
            std::vector<double>& v = word == "receptor_lj" ? p.rec_lj : p.lig_lj;
            v.resize((size_t)n * per);
            for (double& x : v)
                if (!(in >> x)) die("truncated LJ parameters in " + path);
        } else if (word == "ace") {
            if (!(in >> p.n_types) || p.n_types < 1) die("bad ace size in " + path);
            p.ace.resize((size_t)p.n_types * p.n_types);
            for (double& v : p.ace)
                if (!(in >> v)) die("truncated ace matrix in " + path);
        } else if (word == "receptor_frame" || word == "ligand_frame") {
            double* f = word == "receptor_frame" ? p.rec_frame : p.lig_frame;
            for (int i = 0; i < 12; ++i)
                if (!(in >> f[i])) die("truncated frame in " + path);
            (word == "receptor_frame" ? p.has_rec_frame : p.has_lig_frame) = true;
        } else {
            die("unknown section '" + word + "' in " + path);
        }
    }
    return p;
}

// loadRotationalGrid (Geom/rotational_grid.hpp:25-64) + eulerAngToRotMatr
// (Geom/euler.hpp:38-52); a short final read repeats the last angles
std::vector<double> read_rotations(const std::string& path) {
    std::ifstream in(path);
    if (!in.good()) die("cannot open rotations file " + path);
    int n = -1;
    in >> n;
    if (n <= 0) die("no rotation count in " + path);
    in.ignore(1000, '\n');
    const double pi = 4.0 * std::atan(1.0);
    const double deg = pi / 180.0;
    std::vector<double> rot;
    double a[3] = {0, 0, 0};
    for (int i = 0; i < n; ++i) {
        double b[3];
        if (in >> b[0] >> b[1] >> b[2]) std::memcpy(a, b, sizeof(a));
        const double x = a[0] * deg, y = a[1] * deg, z = a[2] * deg;
        const double sa = std::sin(x), ca = std::cos(x), sb = std::sin(y), cb = std::cos(y), sg = std::sin(z),
                     cg = std::cos(z);
        const double m[9] = {cg * ca,           cg * sa,           -sg,
                             sb * sg * ca - cb * sa, sb * sg * sa + cb * ca, cg * sb,
                             cb * sg * ca + sb * sa, cb * sg * sa - sb * ca, cg * cb};
        rot.insert(rot.end(), m, m + 9);
    }
    return rot;
}

std::string arg(std::map<std::string, std::string>& a, const char* k, bool required = true) {
    auto it = a.find(k);
    if (it == a.end()) {
        if (required) die(std::string("missing ") + k);
        return "";
    }
    return it->second;
}

int run_rot_scan(std::map<std::string, std::string>& a) {
    const auto opt = read_json_scalars(arg(a, "--options"));
    const Pair p = read_pair(arg(a, "--molforce-params"));
    const std::vector<double> all_rot = read_rotations(opt.count("anglesFile") ? opt.at("anglesFile")
                                                                              : arg(a, "--angles-file"));
    const int n_all = (int)(all_rot.size() / 9);
    int start = std::atoi(arg(a, "--fft-rot-grid-start").c_str());
    int end = std::atoi(arg(a, "--fft-rot-grid-end").c_str());
    if (start < 0 || start >= n_all) die("Rotation start index is out of bound");
    if (end < start) die("rotation end index is out of bound");
    end = std::min(end, n_all);

    fftdock_config cfg;
    fftdock_config_init(&cfg);
    cfg.grid_step = num(opt, "gridStep", 1.5);
    cfg.peaks_per_rot = (int)num(opt, "maxNTrans", 10);
    cfg.max_trans_inp = (int)num(opt, "maxNTransInp", cfg.peaks_per_rot * 100.0);
    cfg.max_val_corr = num(opt, "maxValCorr", 0.0);
    cfg.rot_batch = (int)num(opt, "rotBatch", 64);
    // Worker::init (docking_app.hpp:369-382)
    cfg.cluster_trans = num(opt, "doClusterTranslations", 0.0) != 0.0 ? 1 : 0;
    cfg.cluster_radius = num(opt, "clusterRadiusTrans", 5.0);
    const std::string corder = opt.count("clusterOrder") ? opt.at("clusterOrder") : "reference";
    if (corder != "reference" && corder != "best_first") die("clusterOrder must be reference or best_first");
    cfg.cluster_order = corder == "best_first" ? FFTDOCK_CLUSTER_ORDER_BEST_FIRST : FFTDOCK_CLUSTER_ORDER_REFERENCE;
    // potentialName "ljComp" / "ljAvg" select the reference's own potentials
    // (docking_app.hpp:52-66); termSet selects this library's shape terms
    const std::string pot = opt.count("potentialName") ? opt.at("potentialName") : "";
    const std::string terms = opt.count("termSet") ? opt.at("termSet") : (p.n_types ? "shape_ace" : "shape");
    cfg.term_set = terms == "shape" ? FFTDOCK_TERMS_SHAPE : FFTDOCK_TERMS_SHAPE_ACE;
    if (pot == "ljComp") cfg.term_set = FFTDOCK_TERMS_LJ_COMP;
    if (pot == "ljAvg") cfg.term_set = FFTDOCK_TERMS_LJ_AVG;
    const bool lj = cfg.term_set == FFTDOCK_TERMS_LJ_COMP || cfg.term_set == FFTDOCK_TERMS_LJ_AVG;
    cfg.lj_cut = num(opt, "cutOffFft", 9.0);
    cfg.lj_mix = (int)num(opt, "ljMix", 1.0);
    if (lj && (p.rec_lj.size() != 3 * p.rec_type.size() || p.lig_lj.size() != 2 * p.lig_type.size()))
        die("the LJ potentials need receptor_lj and ligand_lj sections for every atom");
    cfg.n_types = p.n_types ? p.n_types : 18;
    cfg.ace_matrix = p.ace.empty() ? nullptr : p.ace.data();
    int n = (int)num(opt, "gridN", 0);
    if (n <= 0) {
        // the reference's rule: padded receptor box (docking_molstruct.hpp:
        // 232-244), FFTW-friendly size per axis (docking_fft.hpp:541-553),
        // each axis sized on its own
        double lig = 0.0;
        const size_t nl = p.lig_xyz.size() / 3;
        for (size_t i = 0; i < nl; ++i)
            for (size_t j = i + 1; j < nl; ++j) {
                double d2 = 0;
                for (int k = 0; k < 3; ++k) d2 += std::pow(p.lig_xyz[3 * i + k] - p.lig_xyz[3 * j + k], 2);
                lig = std::max(lig, d2);
            }
        const double pad = (cfg.grid_step * 2.0 + std::sqrt(lig) / 2.0) + num(opt, "cutOffFft", 9.0);
        int32_t dims[3] = {0, 0, 0};
        for (int k = 0; k < 3; ++k) {
            double lo = INFINITY, hi = -INFINITY;
            for (size_t i = 0; i < p.rec_xyz.size() / 3; ++i) {
                lo = std::min(lo, p.rec_xyz[3 * i + k]);
                hi = std::max(hi, p.rec_xyz[3 * i + k]);
            }
            lo -= pad;
            hi += pad;
            // findBestSize(Geom(h, lo).toLogical(hi))
            const double zero_h = lo - cfg.grid_step;
            fftdock_find_best_size((int32_t)((hi - zero_h) / cfg.grid_step) - 1, &dims[k]);
        }
        if (!fftdock_supported_dims(dims[0], dims[1], dims[2]))
            die("the receptor box needs a grid of " + std::to_string(dims[0]) + " x " + std::to_string(dims[1]) +
                " x " + std::to_string(dims[2]) + ", beyond the supported sizes");
        cfg.grid_nx = dims[0];
        cfg.grid_ny = dims[1];
        cfg.grid_nz = dims[2];
        n = dims[0];
    }
    cfg.grid_n = n;

    fftdock_ctx* ctx = nullptr;
    int rc = fftdock_create(&cfg, &ctx);
    if (rc) die(std::string("create: ") + fftdock_last_error(ctx), 2);
    if (lj) {
        const size_t nr = p.rec_type.size(), nl = p.lig_type.size();
        std::vector<double> rs(nr), re(nr), ra(nr), ls(nl), le(nl);
        for (size_t i = 0; i < nr; ++i) {
            rs[i] = p.rec_lj[3 * i];
            re[i] = p.rec_lj[3 * i + 1];
            ra[i] = p.rec_lj[3 * i + 2];
        }
        for (size_t i = 0; i < nl; ++i) {
            ls[i] = p.lig_lj[2 * i];
            le[i] = p.lig_lj[2 * i + 1];
        }
        rc = fftdock_set_pair_lj(ctx, (int32_t)nr, p.rec_xyz.data(), rs.data(), re.data(), ra.data(), (int32_t)nl,
                                 p.lig_xyz.data(), ls.data(), le.data());
    } else {
        rc = fftdock_set_receptor(ctx, (int32_t)p.rec_type.size(), p.rec_xyz.data(), p.rec_type.data());
        if (!rc) rc = fftdock_set_ligand(ctx, (int32_t)p.lig_type.size(), p.lig_xyz.data(), p.lig_type.data());
    }
    const int nr = end - start;
    std::vector<fftdock_peak> peaks((size_t)std::max(nr, 1) * cfg.peaks_per_rot);
    std::vector<int32_t> npk(std::max(nr, 1));
    if (!rc) rc = fftdock_scan(ctx, nr, all_rot.data() + (size_t)start * 9, start, peaks.data(), npk.data());
    if (rc) {
        const std::string msg = fftdock_last_error(ctx);
        fftdock_destroy(ctx);
        die("scan: " + msg, 2);
    }
    fftdock_destroy(ctx);
    rc = fftdock_write_scan_records(arg(a, "--fft-rot-scan-res").c_str(), nr, all_rot.data() + (size_t)start * 9,
                                    cfg.peaks_per_rot, peaks.data(), npk.data(), 0);
    if (rc) die("cannot write " + arg(a, "--fft-rot-scan-res"), 2);
    return 0;
}

int run_gather(std::map<std::string, std::string>& a) {
    const auto opt = read_json_scalars(arg(a, "--options"));
    const int max_matches = (int)num(opt, "maxNRigidMatches", 20000);
    std::vector<fftdock_pose> poses(std::max(max_matches, 1));
    int32_t n = 0;
    int rc = fftdock_gather_list(arg(a, "--fft-rot-scan-list").c_str(), max_matches, poses.data(), &n);
    if (rc) die("gather failed reading the scan records", 2);
    const double *rf = nullptr, *lf = nullptr;
    Pair p;
    const std::string mf = arg(a, "--molforce-params", false);
    if (!mf.empty()) {
        p = read_pair(mf);
        if (p.has_rec_frame) rf = p.rec_frame;
        if (p.has_lig_frame) lf = p.lig_frame;
    }
    const bool text = arg(a, "--fft-res-format", false) == "t";
    rc = fftdock_write_rigid(arg(a, "--fft-res").c_str(), poses.data(), n, rf, lf, text ? 1 : 0);
    if (rc) die("cannot write " + arg(a, "--fft-res"), 2);
    return 0;
}

}  // namespace

int main(int argc, char** argv) {
    std::map<std::string, std::string> a;
    for (int i = 1; i < argc; ++i) {
        const std::string k = argv[i];
        if (k == "-h" || k == "--help") {
            std::printf(
                "usage: fftdock-scan --task rot-scan|gather --options FILE [--molforce-params PAIR]\n"
                "       rot-scan: --fft-rot-grid-start S --fft-rot-grid-end E --fft-rot-scan-res OUT\n"
                "       gather:   --fft-rot-scan-list LIST --fft-res OUT [--fft-res-format b|t]\n");
            return 0;
        }
        if (k.rfind("--", 0) != 0 || i + 1 >= argc) die("bad argument " + k);
        a[k] = argv[++i];
    }
    const std::string task = arg(a, "--task");
    if (task == "rot-scan") return run_rot_scan(a);
    if (task == "gather") return run_gather(a);
    die("unknown task " + task);
}
