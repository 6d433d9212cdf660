// bgk2d_main.cpp -- host driver over the C ABI, in place of the reference's Fortran driver.
//
// Reads the reference's `bgk.input` namelist (SRC/input.F90:44-65), sets the case up like
// SRC/initialize.F90, runs the time loop of SRC/bgk2d.F90:92-113 (boundaries, propagation and
// collision are one fused step on the device) and writes the reference's text outputs at its
// diagnostic cadence (SRC/diagnostic.F90): diagno.dat, probe.dat, u_med.dat, prof_i.dat, prof_j.dat,
// tec_ob.00000000.vtk and obstacle.dat for obstacle cases,
// drag.lift.dat, save.XXXXXXXX.bin checkpoints (Fortran unformatted sequential records, as
// SRC/save_raw.F90), tec_xy/tec_om VTK files (SRC/vtk_xy.binary.F90, SRC/vtk_om.binary.F90, from
// fields computed on the device) and bgk.perf.
//
//   bgk2d_gb300 [--input bgk.input] [--case LDC|TGV|POF|VKS|COU|BFS|MYV] [--prec single|double|mixed2|f16|bf16]
//               [--scheme pingpong|aa|original] [--les 0|1] [--trick1 0|1] [--noshift 0|1]
//               [--forcing-y 0|1] [--obstacle circle|square|half_circle|read[:FILE]] [--dir OUTDIR]
//               [--check-input 0|1]
// `--les 1` stands for the reference's -DLES build (Smagorinsky constant from the namelist key cteS),
// `--trick1 1` for its -DTRICK1 build (lid-cavity boundaries in one merged loop; square LDC only),
// `--noshift 1` for its -DNOSHIFT build (whole populations, not deviations; FP32/FP64 only),
// `--forcing-y 1` for -DFORCING_Y (the POF/MYV body force along y); `--case MYV` is -DMYVERSION.
// `--obstacle` picks the obstacle of an -DOBSTACLE build: the circle (default of VKS), -DSQUARE,
// -DHALF_CIRCLE, or -DREAD, which takes the mask from fort.96 (or FILE).
// `--check-input 1` parses the input, prints the case it describes and exits, without a GPU.
#include <cctype>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include <sys/resource.h>

#include "../../include/bgk2d_gb300.h"

namespace {

std::string fortran_e(double v, int w = 14, int d = 6)
{
    // Fortran Ew.d: 0.ddddddE+xx, right-justified in w columns
    char buf[64];
    if (v == 0.0 || !std::isfinite(v)) {
        if (!std::isfinite(v)) std::snprintf(buf, sizeof(buf), "%*s", w, std::isnan(v) ? "NaN" : (v > 0 ? "Infinity" : "-Infinity"));
        else std::snprintf(buf, sizeof(buf), "%*s", w, "0.000000E+00");
        return buf;
    }
    int e = (int)std::floor(std::log10(std::fabs(v))) + 1;
    double m = v / std::pow(10.0, e);
    char mant[32];
    std::snprintf(mant, sizeof(mant), "%.*f", d, std::fabs(m));
    if (mant[0] == '1') {  // rounding carried to 1.000000
        e += 1;
        m = v / std::pow(10.0, e);
        std::snprintf(mant, sizeof(mant), "%.*f", d, std::fabs(m));
    }
    char s[64];
    std::snprintf(s, sizeof(s), "%s%sE%c%02d", v < 0 ? "-" : "", mant, e < 0 ? '-' : '+', std::abs(e));
    std::snprintf(buf, sizeof(buf), "%*s", w, s);
    return buf;
}

std::map<std::string, std::string> read_namelist(const std::string &path)
{
    std::ifstream f(path);
    std::stringstream ss;
    ss << f.rdbuf();
    std::string t = ss.str();
    for (char &c : t) c = (char)std::tolower((unsigned char)c);  // namelist names ignore case
    for (size_t c = t.find('!'); c != std::string::npos; c = t.find('!', c))  // comments run to end of line
        t.erase(c, t.find('\n', c) == std::string::npos ? std::string::npos : t.find('\n', c) - c);
    std::map<std::string, std::string> kv;
    size_t a = t.find("&parameters");
    if (a == std::string::npos) return kv;
    size_t b = t.find('/', a);
    std::string body = t.substr(a + 11, b - a - 11);
    for (char &c : body)
        if (c == ',' || c == '\n' || c == '\r' || c == '\t') c = ' ';
    std::stringstream bs(body);
    std::string tok, key;
    std::vector<std::string> toks;
    while (bs >> tok) toks.push_back(tok);
    for (size_t i = 0; i < toks.size(); ++i) {
        std::string s = toks[i];
        size_t eq = s.find('=');
        if (eq == std::string::npos) continue;
        std::string k = s.substr(0, eq), v = s.substr(eq + 1);
        if (k.empty() && i > 0) k = toks[i - 1];
        if (v.empty() && i + 1 < toks.size()) v = toks[++i];
        for (char &c : v)
            if (c == 'd') c = 'e';
        kv[k] = v;
    }
    return kv;
}

// the nine (0:l+1, 0:m+1) host planes of a checkpoint (save.XXXXXXXX.bin / restore.bin)
struct Pops {
    int lx, ly, hb;
    std::vector<char> mem;
    void *p[9];
    size_t n;
    Pops(int l, int m, int host_bytes) : lx(l), ly(m), hb(host_bytes)
    {
        n = (size_t)(l + 2) * (m + 2);
        mem.resize(9 * n * hb);
        for (int q = 0; q < 9; ++q) p[q] = mem.data() + q * n * hb;
    }
};

// The profile files of SRC/prof_j.F90:84-85, SRC/prof_i.F90, SRC/probe.F90 and SRC/varm.F90 (u_med.dat),
// from the readers computed on the device (bgk_prof_j, bgk_prof_i, bgk_probe, bgk_varm: the
// reference's arithmetic, in its storage and compute kinds), so that a diagnostic stop moves
// profiles over the host link instead of the nine population planes.
int write_prof_j(bgk_handle *h, int icoord, int ly, FILE *f, int itime)
{
    std::vector<double> u(ly), v(ly), den(ly);
    const int rc = bgk_prof_j(h, icoord, u.data(), v.data(), den.data());
    if (rc) return rc;
    std::fprintf(f, "# t=%7d\n", itime);
    for (int j = 1; j <= ly; ++j)
        std::fprintf(f, "%s %s %s %s \n", fortran_e(j - 0.5).c_str(), fortran_e(u[j - 1]).c_str(),
                     fortran_e(v[j - 1]).c_str(), fortran_e(den[j - 1]).c_str());
    std::fprintf(f, "\n\n");
    return BGK_OK;
}

int write_prof_i(bgk_handle *h, int jcoord, int lx, FILE *f, int itime)
{
    std::vector<double> u(lx), v(lx), den(lx);
    const int rc = bgk_prof_i(h, jcoord, u.data(), v.data(), den.data());
    if (rc) return rc;
    std::fprintf(f, "# t=%7d\n", itime);
    for (int i = 1; i <= lx; ++i)
        std::fprintf(f, "%s %s %s %s \n", fortran_e(i - 0.5).c_str(), fortran_e(u[i - 1]).c_str(),
                     fortran_e(v[i - 1]).c_str(), fortran_e(den[i - 1]).c_str());
    std::fprintf(f, "\n\n");
    return BGK_OK;
}

int write_probe(bgk_handle *h, int i0, int j0, FILE *f, int itime)
{
    double o[3];
    const int rc = bgk_probe(h, i0, j0, o);
    if (rc) return rc;
    std::fprintf(f, "%8d%s %s %s \n", itime, fortran_e(o[0]).c_str(), fortran_e(o[1]).c_str(), fortran_e(o[2]).c_str());
    return BGK_OK;
}

// row means of u, w and rho over i = 1..lx (SRC/varm.F90:49-88, u_med.dat)
int write_varm(bgk_handle *h, int ly, FILE *f, int itime)
{
    std::vector<double> u(ly), w(ly), den(ly);
    const int rc = bgk_varm(h, u.data(), w.data(), den.data());
    if (rc) return rc;
    std::fprintf(f, "# t=%7d\n", itime);
    for (int j = 1; j <= ly; ++j)
        std::fprintf(f, "%5d%s %s %s \n", j, fortran_e(u[j - 1]).c_str(), fortran_e(w[j - 1]).c_str(),
                     fortran_e(den[j - 1]).c_str());
    std::fprintf(f, "\n\n");
    return BGK_OK;
}

// peak resident set size in MB, as SRC/get_mem.c reports it
double max_rss_mb()
{
    struct rusage u;
    getrusage(RUSAGE_SELF, &u);
    return (double)u.ru_maxrss / 1024.0;
}

// Fortran list-directed output of a default real, with gfortran's layout (9 significant digits)
std::string list_real(double v)
{
    char b[64];
    const double a = std::fabs(v);
    if (v == 0.0) std::snprintf(b, sizeof(b), "   0.00000000    ");
    else if (a >= 0.1 && a < 1e8) {
        const int digits = std::max(1, (int)std::floor(std::log10(a)) + 1);
        std::snprintf(b, sizeof(b), "   %.*f    ", 9 - digits, v);
    } else std::snprintf(b, sizeof(b), "   %.8E", v);
    return b;
}

// e14.6 of a value that may be infinite (a section that took no time)
std::string fortran_e_inf(double v) { return std::isfinite(v) ? fortran_e(v) : std::string("      Infinity"); }

// Fortran unformatted sequential record: int32 length, payload, int32 length
void write_record(FILE *f, const void *data, uint32_t bytes)
{
    std::fwrite(&bytes, 4, 1, f);
    std::fwrite(data, 1, bytes, f);
    std::fwrite(&bytes, 4, 1, f);
}

bool read_record(FILE *f, void *data, uint32_t bytes)
{
    uint32_t a = 0, b = 0;
    if (std::fread(&a, 4, 1, f) != 1 || a != bytes) return false;
    if (std::fread(data, 1, bytes, f) != bytes) return false;
    return std::fread(&b, 4, 1, f) == 1 && b == bytes;
}

// Big-endian float32 stream (Fortran access='STREAM', CONVERT="BIG_ENDIAN")
void write_be(FILE *f, const float *v, size_t n)
{
    std::vector<unsigned char> b(4 * n);
    for (size_t i = 0; i < n; ++i) {
        uint32_t u;
        std::memcpy(&u, v + i, 4);
        b[4 * i] = (unsigned char)(u >> 24); b[4 * i + 1] = (unsigned char)(u >> 16);
        b[4 * i + 2] = (unsigned char)(u >> 8); b[4 * i + 3] = (unsigned char)u;
    }
    std::fwrite(b.data(), 1, b.size(), f);
}

// Fortran Aw output of a shorter string: right-justified with leading blanks
std::string fa(const char *s, int w)
{
    std::string t(s);
    return (int)t.size() >= w ? t.substr(0, w) : std::string(w - t.size(), ' ') + t;
}

// tec_xy.XXXXXXXX.vtk and tec_om.XXXXXXXX.vtk as SRC/vtk_xy.binary.F90 and SRC/vtk_om.binary.F90
// write them (serial build: offsets 0), from the fields computed on the device
// with_om = false: tec_xy only (the start-up call of SRC/initialize.F90:119-123)
int write_vtk(bgk_handle *h, const std::string &dir, int itime, int lx, int ly, bool with_om = true)
{
    const size_t n = (size_t)lx * ly, n2 = (size_t)(lx - 2) * (ly - 2);
    std::vector<float> u(n), w(n), rho(n), om(n2), st(n2);
    int rc = bgk_vtk_fields(h, u.data(), w.data(), rho.data(), om.data(), st.data());
    if (rc) return rc;
    auto header = [&](FILE *f, int nx, int ny, int org) {
        std::fprintf(f, "# vtk DataFile Version 2.0\nCampo\nBINARY\nDATASET STRUCTURED_POINTS\n");
        std::fprintf(f, "DIMENSIONS %10d %10d %10d\n", nx, ny, 1);
        std::fprintf(f, "ORIGIN %10d %10d %10d\n", org, org, 1);
        std::fprintf(f, "SPACING %10d %10d %10d\n", 1, 1, 1);
        std::fprintf(f, "POINT_DATA%10d\n", nx * ny);  // (A10,I10) keeps 10 of 'POINT_DATA '
    };
    char name[64];
    std::snprintf(name, sizeof(name), "/tec_xy.%08d.vtk", itime);
    FILE *f = std::fopen((dir + name).c_str(), "wb");
    if (!f) return BGK_E_INVALID;
    header(f, lx, ly, 1);
    std::fprintf(f, "%s\n", fa("VECTORS velocity float", 23).c_str());
    std::vector<float> vec(3 * n, 0.0f);
    for (size_t k = 0; k < n; ++k) { vec[3 * k] = u[k]; vec[3 * k + 1] = w[k]; }
    write_be(f, vec.data(), vec.size());
    std::fprintf(f, "%s\n%s\n", fa("SCALARS w float", 21).c_str(), fa("LOOKUP_TABLE default", 20).c_str());
    write_be(f, w.data(), n);
    std::fprintf(f, "%s\n%s\n", fa("SCALARS u float", 21).c_str(), fa("LOOKUP_TABLE default", 20).c_str());
    write_be(f, u.data(), n);
    std::fprintf(f, "%s\n%s\n", fa("SCALARS rho float", 21).c_str(), fa("LOOKUP_TABLE default", 20).c_str());
    write_be(f, rho.data(), n);
    std::fclose(f);
    if (!with_om) return BGK_OK;
    std::snprintf(name, sizeof(name), "/tec_om.%08d.vtk", itime);
    f = std::fopen((dir + name).c_str(), "wb");
    if (!f) return BGK_E_INVALID;
    header(f, lx - 2, ly - 2, 2);
    std::fprintf(f, "%s\n%s\n", fa("SCALARS vorticity float", 24).c_str(), fa("LOOKUP_TABLE default", 20).c_str());
    write_be(f, om.data(), n2);
    std::fprintf(f, "%s\n%s\n", fa("SCALARS stream float", 25).c_str(), fa("LOOKUP_TABLE default", 20).c_str());
    write_be(f, st.data(), n2);
    std::fclose(f);
    return BGK_OK;
}

// The obstacle outputs of an obstacle build at start-up (SRC/initialize.F90:74-80):
// tec_ob.00000000.vtk, the ASCII rectilinear-grid mask of SRC/vtk_obstacle.F90, and
// obstacle.dat, the `i j obs` list of SRC/w.obs.F90.  Their numbers are list-directed output,
// written with gfortran's widths: integers in 12 columns, the default-real mask values as
// "   0.00000000    ".
int write_obstacle_files(bgk_handle *h, const std::string &dir, int lx, int ly)
{
    std::vector<int32_t> obs((size_t)lx * ly);
    int32_t bbox[5];
    int rc = bgk_get_obs(h, obs.data(), bbox);
    if (rc) return rc;
    if (bbox[4] == 0) return BGK_OK;  // no obstacle cell: not an obstacle build
    FILE *f = std::fopen((dir + "/tec_ob.00000000.vtk").c_str(), "w");
    if (!f) return BGK_E_INVALID;
    std::fprintf(f, "# vtk DataFile Version 2.0\nCampo\nASCII\nDATASET RECTILINEAR_GRID\n");
    std::fprintf(f, "DIMENSIONS %10d %10d%s\n", lx, ly, fa(" 1", 3).c_str());
    std::fprintf(f, "X_COORDINATES %10d double\n", lx);
    for (int i = 1; i <= lx; ++i) std::fprintf(f, "%12d\n", i);
    std::fprintf(f, "Y_COORDINATES %10d double\n", ly);
    for (int j = 1; j <= ly; ++j) std::fprintf(f, "%12d\n", j);
    std::fprintf(f, "Z_COORDINATES %10d double\n%12d\n", 1, 1);
    std::fprintf(f, "%s%10d\n", fa("POINT_DATA ", 10).c_str(), lx * ly);
    std::fprintf(f, "%s\n%s\n", fa("SCALARS obs float", 21).c_str(), fa("LOOKUP_TABLE default", 20).c_str());
    for (int j = 0; j < ly; ++j)
        for (int i = 0; i < lx; ++i) std::fprintf(f, "   %.8f    \n", (double)obs[(size_t)i + (size_t)j * lx]);
    std::fclose(f);
    f = std::fopen((dir + "/obstacle.dat").c_str(), "w");
    if (!f) return BGK_E_INVALID;
    for (int j = 1; j <= ly; ++j)
        for (int i = 1; i <= lx; ++i) std::fprintf(f, "%12d%12d%12d\n", i, j, obs[(size_t)(i - 1) + (size_t)(j - 1) * lx]);
    std::fclose(f);
    return BGK_OK;
}

// The obstacle file of the reference's READ build (SRC/build.obs.F90:148-168, unit 96): one
// list-directed record `x y obs` per cell, i fastest within each row j; x and y are read and
// dropped, and a cell is an obstacle where obs is 1.  The reference reads a hardwired 414 x 414
// block ("WARNING: hardwired parameters"); this reads the domain's lx x ly cells, and rejects a
// file with fewer records or a non-integer obs.
bool read_obstacle_file(const std::string &path, int lx, int ly, std::vector<int32_t> &mask, int &nobs)
{
    std::ifstream f(path);
    if (!f) return false;
    auto next = [&f](std::string &t) -> bool {  // values separated by blanks, newlines or commas
        t.clear();
        char c;
        while (f.get(c)) {
            if (std::isspace((unsigned char)c) || c == ',') {
                if (!t.empty()) return true;
            } else {
                t.push_back(c);
            }
        }
        return !t.empty();
    };
    mask.assign((size_t)lx * (size_t)ly, 0);
    nobs = 0;
    std::string x, y, o;
    for (int j = 0; j < ly; ++j)
        for (int i = 0; i < lx; ++i) {
            if (!next(x) || !next(y) || !next(o)) return false;
            char *end = nullptr;
            const long v = std::strtol(o.c_str(), &end, 10);
            if (end == o.c_str() || *end != '\0') return false;
            mask[(size_t)i + (size_t)j * lx] = (int32_t)v;
            nobs += v == 1;
        }
    return true;
}

int die(const char *what, int rc)
{
    std::fprintf(stderr, "bgk2d_gb300: %s failed (status %d)\n", what, rc);
    return 1;
}

}  // namespace

int main(int argc, char **argv)
{
    std::string input = "bgk.input", tcase = "LDC", prec = "single", scheme = "pingpong", dir = ".", les = "0";
    std::string check = "0", trick1 = "0", noshift = "0", forcing_y = "0", obstacle;
    const auto bad = [](const char *what, const std::string &v) {
        std::fprintf(stderr, "bgk2d_gb300: bad %s '%s'\n", what, v.c_str());
        return 2;
    };
    if (argc % 2 == 0) return bad("option (no value)", argv[argc - 1]);
    for (int i = 1; i + 1 < argc; i += 2) {
        std::string k = argv[i], v = argv[i + 1];
        if (k == "--input") input = v;
        else if (k == "--case") tcase = v;
        else if (k == "--prec") prec = v;
        else if (k == "--scheme") scheme = v;
        else if (k == "--dir") dir = v;
        else if (k == "--les") les = v;
        else if (k == "--trick1") trick1 = v;
        else if (k == "--noshift") noshift = v;
        else if (k == "--forcing-y") forcing_y = v;
        else if (k == "--obstacle") obstacle = v;
        else if (k == "--check-input") check = v;
        else return bad("option", k);
    }
    if (prec != "single" && prec != "double" && prec != "mixed2" && prec != "f16" && prec != "bf16")
        return bad("--prec", prec);
    if (scheme != "pingpong" && scheme != "aa" && scheme != "original") return bad("--scheme", scheme);
    if (les != "0" && les != "1") return bad("--les", les);
    if (trick1 != "0" && trick1 != "1") return bad("--trick1", trick1);
    if (noshift != "0" && noshift != "1") return bad("--noshift", noshift);
    if (forcing_y != "0" && forcing_y != "1") return bad("--forcing-y", forcing_y);
    if (check != "0" && check != "1") return bad("--check-input", check);
    const bool obs_read = obstacle == "read" || obstacle.rfind("read:", 0) == 0;
    if (!obstacle.empty() && !obs_read && obstacle != "circle" && obstacle != "square" && obstacle != "half_circle")
        return bad("--obstacle", obstacle);
    auto kv = read_namelist(input);
    if (kv.empty()) { std::fprintf(stderr, "bgk2d_gb300: no &parameters namelist in %s\n", input.c_str()); return 1; }
    auto geti = [&](const char *k, int d) { return kv.count(k) ? std::atoi(kv[k].c_str()) : d; };
    auto getd = [&](const char *k, double d) { return kv.count(k) ? std::atof(kv[k].c_str()) : d; };
    const int lx = geti("lx", 0), ly = geti("ly", 0), itfin = geti("itfin", 0);
    const int ivtim = geti("ivtim", 1 << 30), isignal = geti("isignal", 1 << 30), itsave = geti("itsave", 1 << 30);
    const int icheck = geti("icheck", 1 << 30), irestart = geti("irestart", 0), init_v = geti("init_v", 0);

    bgk_case_desc d;
    bgk_default_desc(&d);
    d.lx = lx;
    d.ly = ly;
    d.ipad = geti("ipad", 0);
    d.jpad = geti("jpad", 0);
    d.svisc = getd("svisc", 0.1);
    d.u0 = getd("u0", 0.1);
    d.radius = geti("radius", 16);
    d.les = les == "1";
    d.trick1 = trick1 == "1";
    d.noshift = noshift == "1";
    d.force_y = forcing_y == "1";
    d.cte_s = getd("ctes", 0.1);
    d.scheme = scheme == "aa" ? BGK_SCHEME_AA : scheme == "original" ? BGK_SCHEME_ORIGINAL : BGK_SCHEME_PINGPONG;
    if (prec == "double") { d.storage = BGK_STORE_F64; d.compute = BGK_COMPUTE_F64; }
    else if (prec == "mixed2") { d.storage = BGK_STORE_F32; d.compute = BGK_COMPUTE_F64; }
    else if (prec == "f16") d.storage = BGK_STORE_F16;
    else if (prec == "bf16") d.storage = BGK_STORE_BF16;
    const std::map<std::string, int> cases = {{"LDC", BGK_CASE_LDC}, {"TGV", BGK_CASE_TGV}, {"POF", BGK_CASE_POF},
                                              {"VKS", BGK_CASE_VKS}, {"COU", BGK_CASE_COU}, {"BFS", BGK_CASE_BFS},
                                              {"MYV", BGK_CASE_MYV}};
    if (!cases.count(tcase)) { std::fprintf(stderr, "bgk2d_gb300: unknown case %s\n", tcase.c_str()); return 1; }
    d.tcase = cases.at(tcase);
    std::vector<int32_t> obs_mask;
    int obs_cells = -1;  // obstacle cells of a mask read from a file
    if (obstacle == "circle") d.obstacle = BGK_OBS_CIRCLE;
    else if (obstacle == "square") d.obstacle = BGK_OBS_SQUARE;
    else if (obstacle == "half_circle") d.obstacle = BGK_OBS_HALF_CIRCLE;
    else if (obs_read) {
        const std::string path = obstacle.size() > 5 ? obstacle.substr(5) : "fort.96";
        if (lx < 1 || ly < 1 || !read_obstacle_file(path, lx, ly, obs_mask, obs_cells)) {
            std::fprintf(stderr, "bgk2d_gb300: cannot read %d x %d obstacle records from %s\n", lx, ly, path.c_str());
            return 1;
        }
        d.obstacle = BGK_OBS_MASK;
        d.obs_mask = obs_mask.data();
    }
    // init_v is read but, as in SRC/init.F90 (whose argument is unused), the initial state depends
    // on the case alone: the periodic vortex for TGV, rest flow otherwise
    if (d.tcase == BGK_CASE_TGV) d.init_v = BGK_INIT_TGV_REF;
    (void)init_v;
    if (check == "1") {
        std::printf("case=%s prec=%s scheme=%s les=%d trick1=%d noshift=%d forcing_y=%d lx=%d ly=%d ipad=%d jpad=%d svisc=%.17g u0=%.17g "
                    "ctes=%.17g radius=%d itfin=%d ivtim=%d isignal=%d itsave=%d icheck=%d irestart=%d obstacle=%s obs_cells=%d\n",
                    tcase.c_str(), prec.c_str(), scheme.c_str(), d.les, d.trick1, d.noshift, d.force_y, d.lx, d.ly, d.ipad, d.jpad, d.svisc, d.u0,
                    d.cte_s, d.radius, itfin, ivtim, isignal, itsave, icheck, irestart,
                    obstacle.empty() ? "default" : obs_read ? "read" : obstacle.c_str(), obs_cells);
        return 0;
    }

    const auto t0 = std::chrono::steady_clock::now();
    bgk_handle *h = nullptr;
    int rc = bgk_create(&d, &h);
    if (rc) return die("bgk_create", rc);
    const int hb = d.storage == BGK_STORE_F64 ? 8 : 4;
    Pops pops(lx, ly, hb);
    // one plane per checkpoint record, behind a 4-byte length marker: below 2 GiB.  Longer records
    // would need gfortran's subrecords, which this driver does not write.
    const uint64_t rec_bytes = (uint64_t)pops.n * hb;
    const bool rec_ok = rec_bytes < (1ull << 31);
    const double mem_start = max_rss_mb();  // after the allocations, as SRC/alloca.F90:168
    int itstart = 0;
    if (irestart == 1) {  // SRC/restore_raw.F90
        if (!rec_ok) { std::fprintf(stderr, "bgk2d_gb300: restore.bin planes above 2 GiB are not supported\n"); return 1; }
        FILE *f = std::fopen((dir + "/restore.bin").c_str(), "rb");
        int32_t it = 0;
        bool ok = f && read_record(f, &it, 4);
        for (int q = 0; ok && q < 9; ++q) ok = read_record(f, pops.p[q], (uint32_t)rec_bytes);
        if (f) std::fclose(f);
        if (!ok) { std::fprintf(stderr, "bgk2d_gb300: cannot read restore.bin\n"); return 1; }
        itstart = it;
        if ((rc = bgk_upload(h, pops.p, lx + 2))) return die("bgk_upload", rc);
    }
    if ((rc = write_obstacle_files(h, dir, lx, ly))) return die("obstacle files", rc);
    FILE *fdiag = std::fopen((dir + "/diagno.dat").c_str(), "w");
    FILE *fprobe = std::fopen((dir + "/probe.dat").c_str(), "w");
    FILE *fpi = std::fopen((dir + "/prof_i.dat").c_str(), "w");
    FILE *fpj = std::fopen((dir + "/prof_j.dat").c_str(), "w");
    FILE *fumed = std::fopen((dir + "/u_med.dat").c_str(), "w");  // SRC/setup.F90:127-128
    FILE *fdrag = d.tcase == BGK_CASE_VKS ? std::fopen((dir + "/drag.lift.dat").c_str(), "w") : nullptr;
    if (!fdiag || !fprobe || !fpi || !fpj || !fumed || (d.tcase == BGK_CASE_VKS && !fdrag)) {
        std::fprintf(stderr, "bgk2d_gb300: cannot write the output files in %s\n", dir.c_str());
        return 1;
    }
    // probe, varm, prof_i and prof_j in the order of SRC/diagnostic.F90:70-82, computed on the device
    auto readers = [&](int itime, bool with_probe) -> int {
        int r = with_probe ? write_probe(h, lx / 2, ly / 2, fprobe, itime) : BGK_OK;
        if (!r) r = write_varm(h, ly, fumed, itime);
        if (!r) r = write_prof_i(h, ly / 2, lx, fpi, itime);
        if (!r) r = write_prof_j(h, lx / 2, ly, fpj, itime);
        return r;
    };
    // SRC/diagnostic.F90:70-82 at every icheck (diagno, probe, varm, prof_i, prof_j, draglift);
    // SRC/bgk2d.F90:122-125 once after the loop (diagno, varm, prof_i, prof_j)
    auto diagnostic = [&](int itime, bool final_call) -> int {
        double dg[4];
        int r = bgk_diagno(h, BGK_DIAGNO_REFERENCE, dg);  // the reference's own sums (diagno.dat)
        if (r && r != BGK_E_NUMERIC) return r;
        std::fprintf(fdiag, "%8d%s %s %s %s \n", itime, fortran_e(dg[0]).c_str(), fortran_e(dg[1]).c_str(),
                     fortran_e(dg[2]).c_str(), fortran_e(dg[3]).c_str());
        std::fflush(fdiag);
        if ((r = readers(itime, !final_call))) return r;
        if (fdrag && !final_call) {
            double fl[2];
            if ((r = bgk_draglift_reference(h, fl))) return r;  // the reference's own sums
            std::fprintf(fdrag, " %12d %24.16E %24.16E\n", itime, fl[0], fl[1]);
        }
        return BGK_OK;
    };
    if (irestart != 1) {  // SRC/initialize.F90:116-123 writes the initial profiles and velocity field
        if ((rc = readers(0, false))) return die("profiles", rc);
        if (lx > 2 && ly > 2 && (rc = write_vtk(h, dir, 0, lx, ly, false))) return die("vtk", rc);
    }
    const auto t1 = std::chrono::steady_clock::now();
    auto since = [](std::chrono::steady_clock::time_point a) {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - a).count();
    };
    // section times of SRC/finalize.F90: the fused step (boundaries, streaming and collision)
    // counts as collision time; VTK files and checkpoints as I/O; diagnostics as diagno
    double t_last = 0, t_coll = 0, t_dg = 0, t_io = 0, mem_stop = mem_start;
    int itime = itstart;
    while (itime < itfin) {
        // advance to the next diagnostic, save or signal step
        int next = itfin;
        for (int every : {icheck, itsave, isignal, ivtim})
            if (every > 0) next = std::min(next, (itime / every + 1) * every);
        auto ts = std::chrono::steady_clock::now();
        if ((rc = bgk_step(h, next - itime)) || (rc = bgk_sync(h))) return die("bgk_step", rc);
        t_coll += since(ts);
        itime = next;
        ts = std::chrono::steady_clock::now();
        if (itime % ivtim == 0 && lx > 2 && ly > 2 && (rc = write_vtk(h, dir, itime, lx, ly)))  // SRC/diagnostic.F90:32-57
            return die("vtk", rc);
        t_io += since(ts);
        ts = std::chrono::steady_clock::now();
        if (itime % icheck == 0 && (rc = diagnostic(itime, false))) return die("diagnostic", rc);
        t_dg += since(ts);
        ts = std::chrono::steady_clock::now();
        if (itime % itsave == 0) {  // SRC/save_raw.F90
            if ((rc = bgk_download(h, pops.p, lx + 2))) return die("bgk_download", rc);
            char name[64];
            std::snprintf(name, sizeof(name), "/save.%08d.bin", itime);
            if (!rec_ok) { std::fprintf(stderr, "bgk2d_gb300: checkpoint planes above 2 GiB are not supported\n"); return 1; }
            FILE *f = std::fopen((dir + name).c_str(), "wb");
            if (!f) { std::fprintf(stderr, "bgk2d_gb300: cannot write %s%s\n", dir.c_str(), name); return 1; }
            int32_t it = itime;
            write_record(f, &it, 4);
            for (int q = 0; q < 9; ++q) write_record(f, pops.p[q], (uint32_t)rec_bytes);
            std::fclose(f);
        }
        t_io += since(ts);
        if (itime % isignal == 0) {  // SRC/profile.F90: mean time per step
            const double t = since(t1);
            std::printf(" Iteration %8d  time/step %12.5e s\n", itime, (t - t_last) / isignal);
            t_last = t;
            mem_stop = max_rss_mb();
        }
    }
    bgk_sync(h);
    const double loop = since(t1), init = std::chrono::duration<double>(t1 - t0).count();
    if ((rc = diagnostic(itime, true))) return die("diagnostic", rc);
    mem_stop = max_rss_mb();
    // bgk.perf in the layout and formats of SRC/finalize.F90:34-75 (both clock columns hold the
    // same wall time; move, boundary and obstacle work is inside the fused step)
    const double steps = (double)(itfin - itstart), cells = (double)lx * ly;
    const double mlups = cells * steps / loop / 1e6;
    const char *bar = " #--------------------------------\n";
    FILE *fp = std::fopen((dir + "/bgk.perf").c_str(), "w");
    if (!fp) { std::fprintf(stderr, "bgk2d_gb300: cannot write %s/bgk.perf\n", dir.c_str()); return 1; }
    std::fprintf(fp, "%s # Run info \n%12d%12d\n%s # Time for section \n", bar, lx, ly, bar);
    const struct { const char *name; double t; } sec[] = {
        {"init   time", init}, {"loop   time", loop}, {"coll   time", t_coll}, {"move   time", 0.0},
        {"bc     time", 0.0}, {"I/O    time", t_io}, {"diagno time", t_dg}, {"Obst   time", 0.0}};
    for (const auto &x : sec) std::fprintf(fp, " # %s%s %s \n", x.name, fortran_e(x.t).c_str(), fortran_e(x.t).c_str());
    std::fprintf(fp, " # Check      %s \n", fortran_e(loop - (t_coll + t_io + t_dg)).c_str());
    std::fprintf(fp, "%s # Ratio per section (loop)\n", bar);
    const struct { const char *name; double t; } rat[] = {{"I/O  ", t_io}, {"BC   ", 0.0}, {"Coll ", t_coll},
                                                          {"Diag.", t_dg}, {"Move ", 0.0}, {"Obs  ", 0.0}};
    for (const auto &x : rat) std::fprintf(fp, " # Ratio %s%7.3f %7.3f \n", x.name, x.t / loop, x.t / loop);
    std::fprintf(fp, "%s # Derived (global) metrics \n", bar);
    std::fprintf(fp, " # Mlups      %14.6f \n", mlups);
    // the reference's own expressions (SRC/finalize.F90:61-68), units as it labels them
    std::fprintf(fp, " # coll   Flop%s MFlops\n", fortran_e_inf(130.0 * cells * steps / t_coll / 1e6).c_str());
    std::fprintf(fp, " # coll   BW  %s GB/s\n", fortran_e_inf(72.0 * cells * steps / t_coll / 1e6).c_str());
    std::fprintf(fp, " # move   BW  %s GB/s\n", fortran_e_inf(64.0 * cells * steps / 0.0 / 1e6).c_str());
    std::fprintf(fp, "%s # Memory (task 0) metrics \n", bar);
    std::fprintf(fp, " # Memory (start,stop)%14.6f %14.6f MB\n", mem_start, mem_stop);
    std::fprintf(fp, "%s\n%s", list_real((lx / 1024.0) * (ly / 1024.0) * 9 * 2 * 4).c_str(), bar);
    std::fclose(fp);
    std::printf(" # Mlups      %14.6f \n", mlups);
    for (FILE *f : {fdiag, fprobe, fpi, fpj, fumed})
        if (f) std::fclose(f);
    if (fdrag) std::fclose(fdrag);
    bgk_destroy(h);
    return 0;
}
