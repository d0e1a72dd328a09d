// lsh_compat.cpp -- shallowWater(): the reference's solver entry point
// (src/GPU/ShallowWater.cu:125-486) with its exact argument list, driving the
// GB300 kernels through the C ABI of include/lsh.h.
//
// The loop follows ShallowWater.cu:266-461 on one rank: before every step,
// if a snapshot is due (t >= next save time, tiempo_guardar >= 0) write it --
// the six NetCDF files (netcdf.cu layout) or, with leer_fichero_puntos == 1,
// one line of <prefijo>_eta_puntos.txt -- and advance the save time once;
// eta1 max is updated before every step; stop when t >= tiempo_tot.  Between
// snapshots the steps run on the device without host synchronisation (one
// lsh_run_until per snapshot interval) instead of the reference's blocking dt
// read every step.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/lsh.h"
#include "../../include/lsh_compat.h"

namespace {

struct Host {
    std::vector<double> v[LSH_NVARS];
};

int to_ref_status(int s) {
    if (s == LSH_OK) return 0;
    if (s == LSH_ERR_GPU_OOM) return 1;
    if (s == LSH_ERR_HOST_OOM) return 2;
    return 3;
}

}  // namespace

extern "C" {

int comprobarSoporteCUDA(void) { return lsh_check_device(); }

int shallowWater(lsh_dato_cluster* dc, float xmin, float ymin, float Hmin, char* nombre_bati, char* prefijo,
                 int num_voly_otros, int num_voly_total, float borde_sup, float borde_inf, float borde_izq,
                 float borde_der, float ancho_vol, float alto_vol, float area, float tiempo_tot, float tiempo_guardar,
                 float CFL, float r, float angulo1, float angulo2, float angulo3, float angulo4, float peso, float beta,
                 float mfc, float mf0, float mfs, float vmax1, float vmax2, float gravedad, float epsilon_h, float L,
                 float H, float Q, float T, int num_procs, int id_hebra, double* tiempo, int leer_fichero_puntos,
                 int* indiceVolumenesGuardado, int* posicionesVolumenesGuardado, int num_puntos_guardar) {
    (void)num_voly_otros; (void)area; (void)posicionesVolumenesGuardado;
    if (!dc || !dc->datosVolumenes_1 || !dc->datosVolumenes_2 || num_procs != 1 || id_hebra != 0) return 3;
    const int nx = dc->num_volx, ny = dc->num_voly;
    if (nx < 1 || ny < 1 || num_voly_total != ny) return 3;
    const size_t N = size_t(nx) * ny;

    lsh_params p;
    lsh_params_default(&p);
    p.nx = nx; p.ny = ny;
    p.dx = ancho_vol; p.dy = alto_vol;
    p.borde_sup = borde_sup; p.borde_inf = borde_inf; p.borde_izq = borde_izq; p.borde_der = borde_der;
    p.cfl = CFL; p.r = r;
    p.angle1 = angulo1; p.angle2 = angulo2; p.angle3 = angulo3; p.angle4 = angulo4;
    p.peso = peso; p.beta = beta;
    p.mfc = mfc; p.mf0 = mf0; p.mfs = mfs; p.vmax1 = vmax1; p.vmax2 = vmax2;
    p.gravity = gravedad; p.eps_h = epsilon_h; p.L = L; p.H = H;
    p.track_eta_max = 1;

    Host h;
    try {
        for (auto& a : h.v) a.resize(N);
    } catch (...) {
        return 2;
    }
    const lsh_float4* d1 = dc->datosVolumenes_1 + nx;  // row 0 is the halo row
    const lsh_float4* d2 = dc->datosVolumenes_2 + nx;
    for (size_t c = 0; c < N; ++c) {
        h.v[0][c] = d1[c].x; h.v[1][c] = d1[c].y; h.v[2][c] = d1[c].z;
        h.v[3][c] = d2[c].x; h.v[4][c] = d2[c].y; h.v[5][c] = d2[c].z;
        h.v[6][c] = d1[c].w;
    }
    lsh_ctx* ctx = nullptr;
    int s = lsh_create(&p, -1, &ctx);
    if (s) return to_ref_status(s);
    const double* src[LSH_NVARS];
    double* dst[LSH_NVARS];
    for (int k = 0; k < LSH_NVARS; ++k) { src[k] = h.v[k].data(); dst[k] = h.v[k].data(); }
    double dt0 = 0.0;
    if ((s = lsh_set_state(ctx, src, &dt0))) { lsh_destroy(ctx); return to_ref_status(s); }

    // outputs (ShallowWater.cu:210-234)
    lsh_nc* nc = nullptr;
    FILE* fp = nullptr;
    std::vector<float> fv(N);
    if (leer_fichero_puntos == 0) {
        std::vector<float> xs(nx), ys(ny), bati(N);
        for (int i = 0; i < nx; ++i) xs[i] = (float)(xmin * L + (i + 0.5) * ancho_vol * L);
        for (int j = 0; j < ny; ++j) ys[j] = (float)(ymin * L + (j + 0.5) * alto_vol * L);
        for (size_t c = 0; c < N; ++c) bati[c] = (float)((h.v[6][c] + Hmin) * H);
        const double fac = (Q / H) * std::sqrt((double)L) / std::pow((double)H, 7.0 / 6.0);
        const double rad2deg = 180.0 / 3.14159265358979323846;
        const float ang[4] = {(float)(angulo1 * rad2deg), (float)(angulo2 * rad2deg), (float)(angulo3 * rad2deg),
                              (float)(angulo4 * rad2deg)};
        s = lsh_nc_create(prefijo, nombre_bati, nx, ny, xs.data(), ys.data(), bati.data(), tiempo_tot * T, CFL, r,
                          ang, 0, mfc / L, (float)(mf0 / fac), (float)(mfs / fac), vmax1 * Q / H, vmax2 * Q / H, &nc);
        if (s) { lsh_destroy(ctx); return to_ref_status(s); }
    } else {
        std::string name = std::string(prefijo) + "_eta_puntos.txt";
        fp = std::fopen(name.c_str(), "wt");
        if (!fp) { lsh_destroy(ctx); return 3; }
    }

    // gauge mode: the gauge cells' h1 - H gathered on the device, 8 bytes per
    // gauge per row (ShallowWater.cu:318-331 prints (h1 - H - Hmin) H)
    std::vector<int> gcells;
    std::vector<double> gval;
    if (fp) {
        for (int g = 0; g < num_puntos_guardar; ++g) {
            const int c = indiceVolumenesGuardado ? indiceVolumenesGuardado[g] : -1;
            if (c >= 0 && (size_t)c < N) gcells.push_back(c);
        }
        gval.resize(gcells.size());
    }
    auto snapshot = [&](double t) -> int {
        if (nc) {
            int st = lsh_get_state(ctx, dst);
            if (st) return st;
            std::vector<float> f[6];
            for (auto& a : f) a.resize(N);
            for (size_t c = 0; c < N; ++c) {
                f[0][c] = (float)((h.v[0][c] + h.v[3][c] - h.v[6][c] - Hmin) * H);  // :281
                f[1][c] = (float)(h.v[1][c] * Q);
                f[2][c] = (float)(h.v[2][c] * Q);
                f[3][c] = (float)(h.v[3][c] * H);                                   // :301 (h2, not an elevation)
                f[4][c] = (float)(h.v[4][c] * Q);
                f[5][c] = (float)(h.v[5][c] * Q);
            }
            return lsh_nc_write(nc, (float)(t * T), f[0].data(), f[1].data(), f[2].data(), f[3].data(), f[4].data(),
                                f[5].data());
        }
        if (int st = lsh_get_gauge_eta(ctx, (int)gcells.size(), gcells.data(), gval.data())) return st;
        std::fprintf(fp, "%e", t * T);
        size_t k = 0;
        for (int g = 0; g < num_puntos_guardar; ++g) {
            const int c = indiceVolumenesGuardado ? indiceVolumenesGuardado[g] : -1;
            if (c >= 0 && (size_t)c < N) std::fprintf(fp, " %.8e", (gval[k++] - Hmin) * H);  // :325
            else std::fprintf(fp, " -999");
        }
        std::fprintf(fp, "\n");
        return LSH_OK;
    };

    const auto t0 = std::chrono::steady_clock::now();
    double t = 0.0, dtn = 0.0, next_save = 0.0;
    long long steps = 0;
    while (s == LSH_OK && t < tiempo_tot) {
        if (tiempo_guardar >= 0.0 && t >= next_save) {
            if ((s = snapshot(t))) break;
            next_save += tiempo_guardar;
        }
        const double target = (tiempo_guardar >= 0.0 && next_save < tiempo_tot) ? next_save : (double)tiempo_tot;
        if (t >= target) {
            // a step longer than the save interval: take one step, as the reference does
            if ((s = lsh_step(ctx, 1))) break;
            s = lsh_synchronize(ctx);
        } else {
            long long n = 0;
            s = lsh_run_until(ctx, target, 0, &n);
        }
        if (s == LSH_OK) s = lsh_get_time(ctx, &t, &dtn, &steps);
    }
    const auto t1 = std::chrono::steady_clock::now();
    if (tiempo) *tiempo = std::chrono::duration<double>(t1 - t0).count();

    std::vector<double> em(N), et(N);
    if (s == LSH_OK) s = lsh_get_eta_max(ctx, em.data(), et.data());
    if (s == LSH_OK) s = lsh_get_state(ctx, dst);
    if (nc) {
        for (size_t c = 0; c < N; ++c) fv[c] = (float)((em[c] - Hmin) * H);  // :470
        lsh_nc_close(nc, s == LSH_OK ? fv.data() : nullptr);
    }
    if (fp) std::fclose(fp);
    if (s == LSH_OK) {
        lsh_float4* o1 = dc->datosVolumenes_1 + nx;
        lsh_float4* o2 = dc->datosVolumenes_2 + nx;
        for (size_t c = 0; c < N; ++c) {
            o1[c].x = (float)h.v[0][c]; o1[c].y = (float)h.v[1][c]; o1[c].z = (float)h.v[2][c];
            o2[c].x = (float)h.v[3][c]; o2[c].y = (float)h.v[4][c]; o2[c].z = (float)h.v[5][c];
        }
        if (dc->eta1_maxima)
            for (size_t c = 0; c < N; ++c) { dc->eta1_maxima[c].x = (float)em[c]; dc->eta1_maxima[c].y = (float)(et[c] * T); }
    }
    lsh_destroy(ctx);
    return to_ref_status(s);
}

}  // extern "C"
