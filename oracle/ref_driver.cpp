// ref_driver.cpp -- TEST INFRASTRUCTURE.  Host driver around the reference's
// own FP32 kernels (compiled from their unmodified sources through
// ref_shim.h).  It replays, for one MPI rank, the launch sequence of
// shallowWater() (src/GPU/ShallowWater.cu:236-263 initial dt, 266-461 time
// loop), emulating each launch with host loops over blockIdx / threadIdx.
// Edges of one colour touch disjoint cells, so running the threads of a
// launch one after another gives what the GPU gives.
//
// Built by oracle/build_ref.sh into oracle/_ref/liblsh_ref.so; never part of
// the product, and only used here to pin the FP64 oracle and make golden
// fixtures (tests/golden/make_golden.py).
#include "ref_shim.h"

uint3 threadIdx;
uint3 blockIdx;

#include "Volumen_kernel.cu"  // pulls in Arista_kernel.cu, Matriz.cu, Constantes.hxx

#include <algorithm>
#include <vector>

namespace {

template <class F>
void launch(dim3 grid, dim3 block, F&& body) {
    for (unsigned by = 0; by < grid.y; ++by)
        for (unsigned bx = 0; bx < grid.x; ++bx)
            for (unsigned ty = 0; ty < block.y; ++ty)
                for (unsigned tx = 0; tx < block.x; ++tx) {
                    blockIdx = make_uint3(bx, by, 0);
                    threadIdx = make_uint3(tx, ty, 0);
                    body();
                }
}

int div_up(int a, int b) { return (a % b != 0) ? (a / b + 1) : (a / b); }

}  // namespace

extern "C" {

// Runs `nsteps` steps of the reference scheme on one rank.
//   state: 7 float arrays of nx*ny (h1 q1x q1y h2 q2x q2y H), updated in place
//   dt_trace: nsteps+1 floats (may be NULL): the initial dt, then the dt
//             computed after each step
//   t_out: simulated time after the steps
//   eta_max / eta_time: nx*ny floats each (may be NULL), initialised by the
//             caller (Problema.cxx:542-546) and updated before every step.
// Parameters are those of shallowWater() for one rank (id_hebra 0,
// ultima_hebra 1) with the angles in radians.  angulo2..4 reach the kernels
// only in the Pouliquen build (ref_driver_pouliquen.cpp); the Coulomb law
// reads angulo1 alone (Arista_kernel.cu:11-16).
int lsh_ref_run(int nx, int ny, float* const* state, float borde_sup, float borde_inf, float borde_izq,
                float borde_der, float ancho_vol, float alto_vol, float area, float CFL, float r,
                float angulo1, float angulo2, float angulo3, float angulo4, float peso, float beta, float mfc,
                float mf0, float mfs, float vmax1, float vmax2,
                float gravedad, float epsilon_h, float L, float H, int nsteps, float* dt_trace, float* t_out,
                float* eta_max, float* eta_time) {
    const int N = nx * ny;
    const int id_hebra = 0, ultima_hebra = 1;
    const float ang = angulo1, ang2 = angulo2, ang3 = angulo3, ang4 = angulo4;
    std::vector<float4> tex1(size_t(ny + 2) * nx), tex2(size_t(ny + 2) * nx);
    std::vector<float4> acc1(N), acc2(N);
    std::vector<float> dtv(N);
    std::vector<float2> etam(N);
    for (int i = 0; i < N; ++i) {
        tex1[nx + i] = make_float4(state[0][i], state[1][i], state[2][i], state[6][i]);
        tex2[nx + i] = make_float4(state[3][i], state[4][i], state[5][i], state[6][i]);
        if (eta_max) etam[i] = make_float2(eta_max[i], eta_time ? eta_time[i] : 0.0f);
    }
    texDatosVolumenes_1.data = tex1.data(); texDatosVolumenes_1.width = nx; texDatosVolumenes_1.height = ny + 2;
    texDatosVolumenes_2.data = tex2.data(); texDatosVolumenes_2.width = nx; texDatosVolumenes_2.height = ny + 2;

    // launch geometry, ShallowWater.cu:34-94
    const int ar_ver1 = (nx / 2 + 1) * ny;
    const int ar_ver2 = (nx % 2 == 0) ? nx * ny / 2 : ar_ver1;
    const int ar_hor1 = (ny / 2 + 1) * nx;
    const int ar_hor2 = (ny % 2 == 0) ? nx * ny / 2 : ar_hor1;
    const dim3 blk(NUM_HEBRAS_ANCHO_ARI, NUM_HEBRAS_ALTO_ARI);
    const dim3 gV1(div_up(ar_ver1 / ny, NUM_HEBRAS_ANCHO_ARI), div_up(ny, NUM_HEBRAS_ALTO_ARI));
    const dim3 gV2(div_up(ar_ver2 / ny, NUM_HEBRAS_ANCHO_ARI), div_up(ny, NUM_HEBRAS_ALTO_ARI));
    const dim3 gH1(div_up(nx, NUM_HEBRAS_ANCHO_ARI), div_up(ar_hor1 / nx, NUM_HEBRAS_ALTO_ARI));
    const dim3 gH2(div_up(nx, NUM_HEBRAS_ANCHO_ARI), div_up(ar_hor2 / nx, NUM_HEBRAS_ALTO_ARI));
    const dim3 gCom(div_up(nx, NUM_HEBRAS_ANCHO_ARI_COM), 1), bCom(NUM_HEBRAS_ANCHO_ARI_COM, 2);
    const dim3 gDT(div_up(N, NUM_HEBRAS_VOL), 1), bDT(NUM_HEBRAS_VOL, 1);
    const dim3 gEst(div_up(nx, NUM_HEBRAS_ANCHO_EST), div_up(ny, NUM_HEBRAS_ALTO_EST));
    const dim3 bEst(NUM_HEBRAS_ANCHO_EST, NUM_HEBRAS_ALTO_EST);
    float4* a1 = acc1.data();
    float4* a2 = acc2.data();

    auto fmin_all = [&]() {
        float m = 1e30f;  // obtenerMinimoReduccion's host fold
        for (int i = 0; i < N; ++i) m = std::min(m, dtv[i]);
        return m;
    };

    // initial dt (ShallowWater.cu:236-263)
    launch(gH1, blk, [&] { procesarAristasDeltaTInicialGPU(nx, ny, N, borde_sup, borde_inf, ancho_vol, r, a1, gravedad, epsilon_h, 3, id_hebra, ultima_hebra); });
    launch(gH2, blk, [&] { procesarAristasDeltaTInicialGPU(nx, ny, N, borde_sup, borde_inf, ancho_vol, r, a1, gravedad, epsilon_h, 4, id_hebra, ultima_hebra); });
    launch(gV1, blk, [&] { procesarAristasDeltaTInicialGPU(nx, ny, N, borde_izq, borde_der, alto_vol, r, a1, gravedad, epsilon_h, 1, id_hebra, ultima_hebra); });
    launch(gV2, blk, [&] { procesarAristasDeltaTInicialGPU(nx, ny, N, borde_izq, borde_der, alto_vol, r, a1, gravedad, epsilon_h, 2, id_hebra, ultima_hebra); });
    launch(gDT, bDT, [&] { obtenerDeltaTVolumenesGPU(a1, dtv.data(), N, area, CFL); });
    float delta_T = fmin_all();
    if (dt_trace) dt_trace[0] = delta_T;
    std::fill(acc1.begin(), acc1.end(), make_float4(0, 0, 0, 0));

    float t = 0.0f;
    for (int it = 0; it < nsteps; ++it) {
        if (eta_max) launch(gEst, bEst, [&] { actualizarEta1MaximaGPU(etam.data(), nx, ny, t); });
        launch(gH1, blk, [&] { procesarAristasNoComGPU(nx, ny, N, borde_sup, borde_inf, ancho_vol, area, r, delta_T, ang, ang2, ang3, ang4, peso, beta, a1, a2, gravedad, epsilon_h, L, H, 3, id_hebra, ultima_hebra); });
        launch(gCom, bCom, [&] { procesarAristasComGPU(nx, ny, N, borde_sup, borde_inf, ancho_vol, area, r, delta_T, ang, ang2, ang3, ang4, peso, beta, a1, a2, gravedad, epsilon_h, L, H, 3, id_hebra, ultima_hebra); });
        launch(gH2, blk, [&] { procesarAristasGPU(nx, ny, N, borde_sup, borde_inf, ancho_vol, area, r, delta_T, ang, ang2, ang3, ang4, peso, beta, a1, a2, gravedad, epsilon_h, L, H, 4, id_hebra, ultima_hebra); });
        launch(gV1, blk, [&] { procesarAristasGPU(nx, ny, N, borde_izq, borde_der, alto_vol, area, r, delta_T, ang, ang2, ang3, ang4, peso, beta, a1, a2, gravedad, epsilon_h, L, H, 1, id_hebra, ultima_hebra); });
        launch(gV2, blk, [&] { procesarAristasGPU(nx, ny, N, borde_izq, borde_der, alto_vol, area, r, delta_T, ang, ang2, ang3, ang4, peso, beta, a1, a2, gravedad, epsilon_h, L, H, 2, id_hebra, ultima_hebra); });
        launch(gEst, bEst, [&] { obtenerEstadoYDeltaTVolumenesGPU(a1, a2, dtv.data(), nx, ny, area, CFL, r, delta_T, ang, ang2, ang3, ang4, mfc, mf0, mfs, vmax1, vmax2, gravedad, epsilon_h, L, H); });
        t += delta_T;
        delta_T = fmin_all();
        if (dt_trace) dt_trace[it + 1] = delta_T;
        for (int i = 0; i < N; ++i) { tex1[nx + i] = acc1[i]; tex2[nx + i] = acc2[i]; }
        std::fill(acc1.begin(), acc1.end(), make_float4(0, 0, 0, 0));
        std::fill(acc2.begin(), acc2.end(), make_float4(0, 0, 0, 0));
    }
    for (int i = 0; i < N; ++i) {
        const float4 v1 = tex1[nx + i], v2 = tex2[nx + i];
        state[0][i] = v1.x; state[1][i] = v1.y; state[2][i] = v1.z;
        state[3][i] = v2.x; state[4][i] = v2.y; state[5][i] = v2.z;
        if (eta_max) { eta_max[i] = etam[i].x; if (eta_time) eta_time[i] = etam[i].y; }
    }
    if (t_out) *t_out = t;
    return 0;
}

}  // extern "C"
