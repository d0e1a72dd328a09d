// lsh_io.cpp -- host-side input and output of the drop-in surface
// (include/lsh_compat.h):
//   * lsh_load_datadat: data.dat / .bat / .ini reader (Problema.cxx:139-549),
//     using C++ istream extraction exactly as the reference does, so its
//     quirks carry over (e.g. reading the gauge flag as int stops at a '.',
//     which is how PValdez/data.dat's "0.9" becomes flag 0 and CFL .9);
//   * a NetCDF classic (CDF-1) writer, written from the published classic
//     format specification (big-endian header of dimensions, attributes and
//     variables, non-record data, then interleaved records), and the six
//     output files of src/GPU/netcdf.cu on top of it.
// Deliberate deviations from the reference, each for a reference bug:
//   * gauge files hold "count" then (x, y) pairs in the grid's own units; the
//     nearest cell is found with obtenerIndicePunto's search (Problema.cxx:8-42)
//     on cell centres.  The reference reads an uninitialised cell count
//     (:301), checks the wrong file (:236), maps lon/lat with hard-coded
//     constants (:326-327) and stores gauge numbers as cell indices for
//     repeated positions (:338-340).

#include <sys/stat.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <new>
#include <string>
#include <vector>

#include "../../include/lsh.h"
#include "../../include/lsh_compat.h"

namespace {

constexpr double kPi = 3.14159265358979323846;

bool file_exists(const std::string& f) {
    struct stat st;
    return ::stat(f.c_str(), &st) == 0;
}

int fail(lsh_problem* p, const std::string& msg) {
    std::snprintf(p->error, sizeof(p->error), "%s", msg.c_str());
    return LSH_ERR_IO;
}

// obtenerIndicePunto (Problema.cxx:8-42): first coordinate >= the point, or
// the one before it when closer; -1 outside.
int nearest_cell(const std::vector<double>& X, const std::vector<double>& Y, double px, double py) {
    const int nx = (int)X.size(), ny = (int)Y.size();
    int i = 0;
    bool found = false;
    while (i < nx && !found) {
        if (X[i] >= px) {
            found = true;
            const int im = (i > 0) ? i - 1 : 0;
            if (std::fabs(px - X[im]) < std::fabs(px - X[i])) i = im;
        } else {
            ++i;
        }
    }
    if (!found) return -1;
    int j = 0;
    found = false;
    while (j < ny && !found) {
        if (Y[j] >= py) {
            found = true;
            const int jm = (j > 0) ? j - 1 : 0;
            if (std::fabs(py - Y[jm]) < std::fabs(py - Y[j])) j = jm;
        } else {
            ++j;
        }
    }
    if (!found) return -1;
    return j * nx + i;
}

}  // namespace

extern "C" {

void lsh_problem_free(lsh_problem* p) {
    if (!p) return;
    for (int k = 0; k < LSH_NVARS; ++k) delete[] p->state[k];
    delete[] p->eta1_max;
    delete[] p->indice_puntos;
    delete p;
}

static int load_impl(const char* path, int law, lsh_problem* P) {
    const std::string fich_ent(path);
    std::string dir;
    std::string::size_type k = fich_ent.find_last_of('/');
    if (k != std::string::npos) dir = fich_ent.substr(0, k) + "/";
    else if ((k = fich_ent.find_last_of('\\')) != std::string::npos) dir = fich_ent.substr(0, k) + "\\";
    if (!file_exists(fich_ent)) return fail(P, "cannot find '" + fich_ent + "'");
    std::ifstream fich(fich_ent.c_str());
    std::string nombre_bati, fich_topo, fich_est, fich_puntos, prefijo;
    int leerDeFichero = 0, nx = 0, ny = 0, leer_puntos = 0, normalizar = 0;
    double xmin = 0, xmax = 0, ymin = 0, ymax = 0;
    std::ifstream fich2;
    fich >> nombre_bati;
    fich >> leerDeFichero;
    if (leerDeFichero == 0) {
        fich >> xmin >> xmax >> ymin >> ymax >> nx >> ny;
    } else {
        fich >> fich_topo >> fich_est;
        fich_topo = dir + fich_topo;
        fich_est = dir + fich_est;
        if (!file_exists(fich_topo)) return fail(P, "cannot find '" + fich_topo + "'");
        if (!file_exists(fich_est)) return fail(P, "cannot find '" + fich_est + "'");
        fich2.open(fich_topo.c_str());
        fich2 >> xmin >> xmax >> ymin >> ymax >> nx >> ny;
        if (fich2.fail()) return fail(P, "malformed header in '" + fich_topo + "'");
    }
    double b_sup, b_inf, b_izq, b_der, t_tot, t_guardar;
    fich >> b_sup >> b_inf >> b_izq >> b_der >> t_tot >> t_guardar;
    fich >> leer_puntos;
    if (leer_puntos == 1) {
        fich >> fich_puntos;
        fich_puntos = dir + fich_puntos;
        if (!file_exists(fich_puntos)) return fail(P, "cannot find '" + fich_puntos + "'");
    }
    double CFL, r, ang[4] = {0, 0, 0, 0}, mfc, mf0, mfs, vmax1, vmax2, L = 1, H = 1, Q = 1, T = 1, g = 9.81;
    fich >> CFL >> r;
    fich >> ang[0];
    if (law == LSH_FRICTION_POULIQUEN) fich >> ang[1] >> ang[2] >> ang[3];
    for (double& a : ang) a *= kPi / 180.0;
    fich >> mfc >> mf0 >> mfs >> vmax1 >> vmax2 >> normalizar;
    if (normalizar != 0) {
        fich >> L >> H;
        Q = std::sqrt(9.81 * std::pow(H, 3.0));
        T = L * H / Q;
        g = 1.0;
        xmin /= L; xmax /= L; ymin /= L; ymax /= L;
        t_tot /= T;
        t_guardar /= T;
        mfc *= L;
        mf0 *= (Q / H) * std::sqrt(L) / std::pow(H, 7.0 / 6.0);
        mfs *= (Q / H) * std::sqrt(L) / std::pow(H, 7.0 / 6.0);
        vmax1 /= Q / H;
        vmax2 /= Q / H;
    }
    fich >> prefijo;
    if (fich.fail()) return fail(P, "malformed data file '" + fich_ent + "'");
    if (nx < 1 || ny < 1) return fail(P, "grid size must be positive");
    const double eps_h = 5e-3 / H;  // Problema.cxx:287
    const double ancho = (xmax - xmin) / nx, alto = (ymax - ymin) / ny;

    lsh_params& p = P->params;
    lsh_params_default(&p);
    p.nx = nx; p.ny = ny; p.dx = ancho; p.dy = alto;
    p.friction_law = law;
    p.borde_sup = b_sup; p.borde_inf = b_inf; p.borde_izq = b_izq; p.borde_der = b_der;
    p.cfl = CFL; p.r = r;
    p.angle1 = ang[0]; p.angle2 = ang[1]; p.angle3 = ang[2]; p.angle4 = ang[3];
    p.mfc = mfc; p.mf0 = mf0; p.mfs = mfs; p.vmax1 = vmax1; p.vmax2 = vmax2;
    p.gravity = g; p.eps_h = eps_h; p.L = L; p.H = H;
    p.peso = 1.0; p.beta = 1.0;  // main.cxx:161
    P->xmin = xmin; P->xmax = xmax; P->ymin = ymin; P->ymax = ymax;
    P->Q = Q; P->T = T;
    P->tiempo_tot = t_tot;
    P->tiempo_guardar = t_guardar;
    P->leer_fichero_puntos = leer_puntos;
    std::snprintf(P->nombre_bati, sizeof(P->nombre_bati), "%s", nombre_bati.c_str());
    std::snprintf(P->prefijo, sizeof(P->prefijo), "%s", prefijo.c_str());

    const size_t N = size_t(nx) * ny;
    for (int v = 0; v < LSH_NVARS; ++v) {
        P->state[v] = new (std::nothrow) double[N];
        if (!P->state[v]) return LSH_ERR_HOST_OOM;
    }
    P->eta1_max = new (std::nothrow) double[N];
    if (!P->eta1_max) return LSH_ERR_HOST_OOM;

    double hmin = 0.0;
    if (leerDeFichero == 0) {
        // the analytic initial condition compiled into the reference
        // (cond_ini.cxx: depth 5 m, both layers empty, at rest)
        for (size_t c = 0; c < N; ++c) {
            P->state[0][c] = 0.0; P->state[1][c] = 0.0; P->state[2][c] = 0.0;
            P->state[3][c] = 0.0; P->state[4][c] = 0.0; P->state[5][c] = 0.0;
            P->state[6][c] = 5.0 / H;
        }
    } else {
        double mn = 1e30;
        for (size_t c = 0; c < N; ++c) {
            double val;
            fich2 >> val;
            val /= H;
            P->state[6][c] = val;
            if (val < mn) mn = val;
        }
        if (fich2.fail()) return fail(P, "bathymetry file '" + fich_topo + "' ends early");
        fich2.close();
        hmin = (mn >= 0.0) ? 0.0 : mn;
        if (hmin < 0.0)
            for (size_t c = 0; c < N; ++c) P->state[6][c] -= hmin;
        std::ifstream fe(fich_est.c_str());
        for (size_t c = 0; c < N; ++c) {
            double W[6];
            fe >> W[0] >> W[1] >> W[2] >> W[3] >> W[4] >> W[5];
            P->state[0][c] = W[0] / H;
            P->state[1][c] = W[1] / Q;
            P->state[2][c] = W[2] / Q;
            P->state[3][c] = W[3] / H;
            P->state[4][c] = W[4] / Q;
            P->state[5][c] = W[5] / Q;
        }
        if (fe.fail()) return fail(P, "initial state file '" + fich_est + "' ends early");
    }
    P->hmin = hmin;
    for (size_t c = 0; c < N; ++c) P->eta1_max[c] = P->state[0][c] + P->state[3][c] - P->state[6][c];

    if (leer_puntos == 1) {
        std::ifstream fp(fich_puntos.c_str());
        int n = 0;
        fp >> n;
        if (fp.fail() || n < 0) return fail(P, "malformed gauge file '" + fich_puntos + "'");
        P->num_puntos_guardar = n;
        P->indice_puntos = new (std::nothrow) int32_t[n > 0 ? n : 1];
        if (!P->indice_puntos) return LSH_ERR_HOST_OOM;
        std::vector<double> X(nx), Y(ny);
        for (int i = 0; i < nx; ++i) X[i] = (xmin + (i + 0.5) * ancho) * L;
        for (int j = 0; j < ny; ++j) Y[j] = (ymin + (j + 0.5) * alto) * L;
        for (int g2 = 0; g2 < n; ++g2) {
            double gx, gy;
            fp >> gx >> gy;
            if (fp.fail()) return fail(P, "gauge file '" + fich_puntos + "' ends early");
            P->indice_puntos[g2] = nearest_cell(X, Y, gx, gy);
        }
    }
    return LSH_OK;
}

int lsh_load_datadat_law(const char* path, int friction_law, lsh_problem** out) {
    if (!out || !path) return LSH_ERR_INVALID;
    *out = nullptr;
    lsh_problem* P = new (std::nothrow) lsh_problem();
    if (!P) return LSH_ERR_HOST_OOM;
    std::memset(P, 0, sizeof(*P));
    const int s = load_impl(path, friction_law, P);
    *out = P;
    return s;
}

int lsh_load_datadat(const char* path, lsh_problem** out) {
    return lsh_load_datadat_law(path, LSH_FRICTION_COULOMB, out);
}

}  // extern "C"

// ---------------------------------------------------------------- NetCDF classic

namespace {

enum { NC_CHAR = 2, NC_FLOAT = 5 };
constexpr uint32_t kNcDimension = 0x0A, kNcVariable = 0x0B, kNcAttribute = 0x0C;

struct NcAtt {
    std::string name;
    int type;
    std::string text;
    std::vector<float> f;
};

struct NcVar {
    std::string name;
    std::vector<int> dims;
    std::vector<NcAtt> atts;
    uint32_t vsize = 0;
    uint32_t begin = 0;
    bool rec = false;
};

// Minimal CDF-1 writer: float variables, text / float attributes, one
// unlimited dimension.
class NcFile {
  public:
    std::vector<std::pair<std::string, uint32_t>> dims;  // length 0 = unlimited
    std::vector<NcAtt> gatts;
    std::vector<NcVar> vars;
    FILE* f = nullptr;
    uint32_t numrecs = 0;
    uint32_t recsize = 0;
    uint32_t data_start = 0;

    int dim(const std::string& name, uint32_t len) {
        dims.emplace_back(name, len);
        return (int)dims.size() - 1;
    }
    int var(const std::string& name, std::vector<int> d) {
        NcVar v;
        v.name = name;
        v.dims = std::move(d);
        v.rec = !v.dims.empty() && dims[v.dims[0]].second == 0;
        vars.push_back(v);
        return (int)vars.size() - 1;
    }
    static NcAtt text(const std::string& n, const std::string& t) { return NcAtt{n, NC_CHAR, t, {}}; }
    static NcAtt flt(const std::string& n, float v) { return NcAtt{n, NC_FLOAT, {}, {v}}; }

    static void be32(std::vector<unsigned char>& b, uint32_t v) {
        b.push_back((v >> 24) & 0xff); b.push_back((v >> 16) & 0xff); b.push_back((v >> 8) & 0xff); b.push_back(v & 0xff);
    }
    static void pad4(std::vector<unsigned char>& b) { while (b.size() % 4) b.push_back(0); }
    static void name(std::vector<unsigned char>& b, const std::string& s) {
        be32(b, (uint32_t)s.size());
        b.insert(b.end(), s.begin(), s.end());
        pad4(b);
    }
    static void atts(std::vector<unsigned char>& b, const std::vector<NcAtt>& a) {
        if (a.empty()) { be32(b, 0); be32(b, 0); return; }
        be32(b, kNcAttribute);
        be32(b, (uint32_t)a.size());
        for (const NcAtt& x : a) {
            name(b, x.name);
            be32(b, (uint32_t)x.type);
            if (x.type == NC_CHAR) {
                be32(b, (uint32_t)x.text.size());
                b.insert(b.end(), x.text.begin(), x.text.end());
                pad4(b);
            } else {
                be32(b, (uint32_t)x.f.size());
                for (float v : x.f) { uint32_t u; std::memcpy(&u, &v, 4); be32(b, u); }
            }
        }
    }
    uint32_t slab_elems(const NcVar& v) const {
        uint32_t n = 1;
        for (size_t i = v.rec ? 1 : 0; i < v.dims.size(); ++i) n *= dims[v.dims[i]].second;
        return n;
    }
    std::vector<unsigned char> header() const {
        std::vector<unsigned char> b = {'C', 'D', 'F', 1};
        be32(b, numrecs);
        if (dims.empty()) { be32(b, 0); be32(b, 0); }
        else {
            be32(b, kNcDimension);
            be32(b, (uint32_t)dims.size());
            for (auto& d : dims) { name(b, d.first); be32(b, d.second); }
        }
        atts(b, gatts);
        if (vars.empty()) { be32(b, 0); be32(b, 0); }
        else {
            be32(b, kNcVariable);
            be32(b, (uint32_t)vars.size());
            for (const NcVar& v : vars) {
                name(b, v.name);
                be32(b, (uint32_t)v.dims.size());
                for (int d : v.dims) be32(b, (uint32_t)d);
                atts(b, v.atts);
                be32(b, NC_FLOAT);
                be32(b, v.vsize);
                be32(b, v.begin);
            }
        }
        return b;
    }
    // lay out offsets, write the header and zero-filled fixed-size data
    bool enddef(const char* path) {
        f = std::fopen(path, "wb");
        if (!f) return false;
        int nrec = 0;
        for (NcVar& v : vars) {
            v.vsize = slab_elems(v) * 4;
            if (v.rec) ++nrec;
        }
        const uint32_t hsize = (uint32_t)header().size();
        uint32_t off = hsize;
        for (NcVar& v : vars)
            if (!v.rec) { v.begin = off; off += v.vsize; }
        data_start = off;
        recsize = 0;
        for (NcVar& v : vars)
            if (v.rec) { v.begin = off + recsize; recsize += v.vsize; }
        // a single record variable is not padded (classic-format rule); all
        // our slabs are float multiples of 4 bytes anyway
        (void)nrec;
        std::vector<unsigned char> h = header();
        std::fwrite(h.data(), 1, h.size(), f);
        std::vector<unsigned char> zeros(data_start - hsize, 0);
        if (!zeros.empty()) std::fwrite(zeros.data(), 1, zeros.size(), f);
        return true;
    }
    static void be_floats(const float* src, size_t n, std::vector<unsigned char>& out) {
        out.resize(n * 4);
        for (size_t i = 0; i < n; ++i) {
            uint32_t u;
            std::memcpy(&u, &src[i], 4);
            out[4 * i] = (u >> 24) & 0xff; out[4 * i + 1] = (u >> 16) & 0xff;
            out[4 * i + 2] = (u >> 8) & 0xff; out[4 * i + 3] = u & 0xff;
        }
    }
    void put(int vi, const float* data) {
        const NcVar& v = vars[vi];
        std::vector<unsigned char> b;
        be_floats(data, slab_elems(v), b);
        std::fseek(f, (long)v.begin, SEEK_SET);
        std::fwrite(b.data(), 1, b.size(), f);
    }
    void put_rec(int vi, uint32_t rec, const float* data) {
        const NcVar& v = vars[vi];
        std::vector<unsigned char> b;
        be_floats(data, slab_elems(v), b);
        std::fseek(f, (long)(v.begin + rec * recsize), SEEK_SET);
        std::fwrite(b.data(), 1, b.size(), f);
        if (rec + 1 > numrecs) {
            numrecs = rec + 1;
            std::vector<unsigned char> n;
            be32(n, numrecs);
            std::fseek(f, 4, SEEK_SET);
            std::fwrite(n.data(), 1, 4, f);
        }
    }
    void close() {
        if (f) std::fclose(f);
        f = nullptr;
    }
};

struct OneFile {
    NcFile nc;
    int time_id = -1, var_id = -1, max_id = -1;
};

}  // namespace

struct lsh_nc {
    OneFile file[6];
    int nx = 0, ny = 0;
    uint32_t rec = 0;
};

extern "C" {

// fgennc / initNC (netcdf.cu:29-335): dims lon, lat [grid_x, grid_y], time;
// variables lon, lat [grid_x, grid_y, bathymetry], time [max_height], field.
int lsh_nc_create(const char* prefix, const char* nombre_bati, int nx, int ny, const float* x, const float* y,
                  const float* bathymetry, float tiempo_tot, float CFL, float r, const float angles_deg[4],
                  int pouliquen, float mfc, float mf0, float mfs, float vmax1, float vmax2, lsh_nc** out) {
    if (!out || !prefix || nx < 1 || ny < 1 || !x || !y || !bathymetry) return LSH_ERR_INVALID;
    *out = nullptr;
    lsh_nc* h = new (std::nothrow) lsh_nc();
    if (!h) return LSH_ERR_HOST_OOM;
    h->nx = nx;
    h->ny = ny;
    static const char* suffix[6] = {"eta1", "q1x", "q1y", "eta2", "q2x", "q2y"};
    static const char* units[6] = {"meters", "meters/second", "meters/second", "meters", "meters/second", "meters/second"};
    static const char* lname[6] = {"Wave amplitude", "Mass flow of water along x", "Mass flow of water along y",
                                   "Sediments", "Mass flow of sediments along x", "Mass flow of sediments along y"};
    const float fill = -1e30f;
    char buf[256];
    for (int k = 0; k < 6; ++k) {
        NcFile& nc = h->file[k].nc;
        const int dlon = nc.dim("lon", nx), dlat = nc.dim("lat", ny);
        int dgx = -1, dgy = -1;
        if (k == 0) { dgx = nc.dim("grid_x", nx); dgy = nc.dim("grid_y", ny); }
        const int dtime = nc.dim("time", 0);
        const int vlon = nc.var("lon", {dlon});
        nc.vars[vlon].atts = {NcFile::text("long_name", "x axis"), NcFile::text("units", "meters")};
        const int vlat = nc.var("lat", {dlat});
        nc.vars[vlat].atts = {NcFile::text("long_name", "y axis"), NcFile::text("units", "meters")};
        int vgx = -1, vgy = -1, vbat = -1;
        if (k == 0) {
            vgx = nc.var("grid_x", {dgx});
            nc.vars[vgx].atts = {NcFile::text("long_name", "Grid x axis"), NcFile::text("units", "meters")};
            vgy = nc.var("grid_y", {dgy});
            nc.vars[vgy].atts = {NcFile::text("long_name", "Grid y axis"), NcFile::text("units", "meters")};
            vbat = nc.var("bathymetry", {dgy, dgx});
            nc.vars[vbat].atts = {NcFile::text("long_name", "Grid bathymetry"), NcFile::text("standard_name", "depth"),
                                  NcFile::text("units", "meters"), NcFile::flt("missing_value", fill),
                                  NcFile::flt("_FillValue", fill)};
        }
        const int vtime = nc.var("time", {dtime});
        nc.vars[vtime].atts = {NcFile::text("long_name", "Time"), NcFile::text("units", "seconds since 1970-01-01")};
        if (k == 0) {
            h->file[k].max_id = nc.var("max_height", {dlat, dlon});
            nc.vars[h->file[k].max_id].atts = {NcFile::text("long_name", "Maximum wave amplitude"),
                                               NcFile::text("units", "meters"), NcFile::flt("missing_value", fill),
                                               NcFile::flt("_FillValue", fill)};
        }
        const int vf = nc.var(suffix[k], {dtime, dlat, dlon});
        nc.vars[vf].atts = {NcFile::text("units", units[k]), NcFile::text("long_name", lname[k]),
                            NcFile::flt("missing_value", fill), NcFile::flt("_FillValue", fill)};
        h->file[k].time_id = vtime;
        h->file[k].var_id = vf;
        nc.gatts.push_back(NcFile::text("Conventions", "CF-1.0"));
        nc.gatts.push_back(NcFile::text("title", "LandSlide-HySEA two-layer model output (GB300 FP64 build)"));
        nc.gatts.push_back(NcFile::text("grid_name", nombre_bati ? nombre_bati : ""));
        nc.gatts.push_back(NcFile::flt("simulation_time", tiempo_tot));
        nc.gatts.push_back(NcFile::flt("CFL", CFL));
        nc.gatts.push_back(NcFile::flt("ratio_of_densities", r));
        if (!pouliquen) {
            nc.gatts.push_back(NcFile::text("friction_law", "Coulomb"));
            std::snprintf(buf, sizeof(buf), "%.4f", angles_deg[0]);
        } else {
            nc.gatts.push_back(NcFile::text("friction_law", "Pouliquen"));
            std::snprintf(buf, sizeof(buf), "%.4f, %.4f, %.4f, %.4f", angles_deg[0], angles_deg[1], angles_deg[2],
                          angles_deg[3]);
        }
        nc.gatts.push_back(NcFile::text("angle_of_repose", buf));
        nc.gatts.push_back(NcFile::flt("friction_between_layers", mfc));
        nc.gatts.push_back(NcFile::flt("friction_water_bottom", mf0));
        nc.gatts.push_back(NcFile::flt("friction_sediments_bottom", mfs));
        nc.gatts.push_back(NcFile::flt("max_speed_water", vmax1));
        nc.gatts.push_back(NcFile::flt("max_speed_sediments", vmax2));
        std::snprintf(buf, sizeof(buf), "%s_%s.nc", prefix, suffix[k]);
        if (!nc.enddef(buf)) {
            for (int j = 0; j <= k; ++j) h->file[j].nc.close();
            delete h;
            return LSH_ERR_IO;
        }
        nc.put(vlon, x);
        nc.put(vlat, y);
        if (k == 0) {
            nc.put(vgx, x);
            nc.put(vgy, y);
            nc.put(vbat, bathymetry);
        }
    }
    *out = h;
    return LSH_OK;
}

// writerecs (netcdf.cu:337-387)
int lsh_nc_write(lsh_nc* h, float time, const float* eta1, const float* q1x, const float* q1y, const float* eta2,
                 const float* q2x, const float* q2y) {
    if (!h) return LSH_ERR_INVALID;
    const float* f[6] = {eta1, q1x, q1y, eta2, q2x, q2y};
    for (int k = 0; k < 6; ++k) {
        if (!f[k]) return LSH_ERR_INVALID;
        h->file[k].nc.put_rec(h->file[k].time_id, h->rec, &time);
        h->file[k].nc.put_rec(h->file[k].var_id, h->rec, f[k]);
    }
    h->rec++;
    return LSH_OK;
}

// closeNC (netcdf.cu:389-411)
int lsh_nc_close(lsh_nc* h, const float* max_height) {
    if (!h) return LSH_ERR_INVALID;
    if (max_height) h->file[0].nc.put(h->file[0].max_id, max_height);
    for (int k = 0; k < 6; ++k) h->file[k].nc.close();
    delete h;
    return LSH_OK;
}

}  // extern "C"
