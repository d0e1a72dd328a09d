// ref_cuda_driver.cpp -- TEST INFRASTRUCTURE.  Runs the reference's own CUDA
// kernels on the GPU: oracle/_ref/ref_kernels.cubin, compiled from the
// reference's unmodified sources by oracle/build_ref.sh (ref_cuda_kernels.cu
// through ref_cuda_shim.h).  It replays, for one MPI rank (id_hebra 0,
// ultima_hebra 1), what shallowWater() does on the device:
//   initial dt      ShallowWater.cu:236-263 (4 wave passes, per-cell dt,
//                   obtenerMinimoReduccion, accumulator reset);
//   each step       ShallowWater.cu:266-461 without output and MPI calls:
//                   actualizarEta1MaximaGPU; the 4 halo-row reads to the host
//                   (cudaMemcpyFromArray, :362-369); the non-halo horizontal
//                   edges; the 4 halo-row writes from the host
//                   (cudaMemcpyToArray, :401-408); the halo edges, the second
//                   horizontal colour and both vertical colours; the state
//                   and per-cell dt kernel; t += dt; the dt min-reduction
//                   (Reduccion_kernel.cu:130-172: reduce6_min, a device-to-
//                   host copy and a host fold); the two texture copy-backs
//                   (:447-450) and the two accumulator memsets (:453-454).
// Launch shapes follow ShallowWater.cu:34-94.  Copies are synchronous, on
// the legacy stream, from pageable host memory, as the reference's are.
// The textures are the shim's plain device arrays of (ny + 2) x nx float4
// (rows 0 and ny + 1 are the halo rows).
//
// Built wherever the cubin is by oracle/build_ref.sh (g++ against libcuda)
// into oracle/_ref/liblsh_ref_cuda.so; bench.py --impl reference
// --ref-build cuda times it.  Never part of the product.
#include <cuda.h>

#include <chrono>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace {

std::string g_err;

#define CU(call)                                                                    \
    do {                                                                            \
        CUresult r_ = (call);                                                       \
        if (r_ != CUDA_SUCCESS) {                                                   \
            const char* s_ = nullptr;                                               \
            cuGetErrorString(r_, &s_);                                              \
            g_err = std::string(#call) + ": " + (s_ ? s_ : "?");                    \
            return 1;                                                               \
        }                                                                           \
    } while (0)

struct TexRef {  // the shim's texture: device pointer, width, height
    unsigned long long data;
    int width;
    int height;
};

struct F4 { float x, y, z, w; };
struct F2 { float x, y; };

// The kernel whose mangled name starts with "_Z" + prefix.
CUfunction find_kernel(const std::vector<CUfunction>& fs, const std::string& prefix) {
    const std::string want = "_Z" + prefix;
    for (CUfunction f : fs) {
        const char* nm = nullptr;
        if (cuFuncGetName(&nm, f) == CUDA_SUCCESS && nm && std::strncmp(nm, want.c_str(), want.size()) == 0)
            return f;
    }
    return nullptr;
}

std::string mangled_prefix(const char* name) { return std::to_string(std::strlen(name)) + name; }

int div_up(int a, int b) { return (a % b != 0) ? (a / b + 1) : (a / b); }

struct Launch {
    CUfunction f;
    unsigned gx, gy, bx, by, smem;
    int run(void** args) const {
        CU(cuLaunchKernel(f, gx, gy, 1, bx, by, 1, smem, nullptr, args, nullptr));
        return 0;
    }
};

}  // namespace

extern "C" {

const char* lsh_ref_cuda_error(void) { return g_err.c_str(); }

// Runs `warmup` untimed steps, then `nsteps` timed steps of the reference on
// device `device`.  state: 7 float arrays of nx*ny (h1 q1x q1y h2 q2x q2y H),
// updated in place; dt_trace (nsteps + 1 floats, may be NULL): the dt at the
// start of the timed steps, then after each; t_out: simulated time after all
// steps; ms_out: wall time of the timed steps in milliseconds.  Angles in
// radians; the parameters are shallowWater()'s (all float).
int lsh_ref_cuda_run(const char* cubin, int device, int nx, int ny, float* const* state, float borde_sup,
                     float borde_inf, float borde_izq, float borde_der, float ancho_vol, float alto_vol, float area,
                     float CFL, float r, float angulo1, float angulo2, float angulo3, float angulo4, float peso,
                     float beta, float mfc, float mf0, float mfs, float vmax1, float vmax2, float gravedad,
                     float epsilon_h, float L, float H, int warmup, int nsteps, float* dt_trace, float* t_out,
                     double* ms_out) {
    CU(cuInit(0));
    CUdevice dev;
    CU(cuDeviceGet(&dev, device));
    CUcontext ctx;
    CU(cuDevicePrimaryCtxRetain(&ctx, dev));
    CU(cuCtxPushCurrent(ctx));
    int status = 0;
    CUmodule mod = nullptr;
    CUdeviceptr d_tex1 = 0, d_tex2 = 0, d_acc1 = 0, d_acc2 = 0, d_dtv = 0, d_eta = 0;
    auto body = [&]() -> int {
        CU(cuModuleLoad(&mod, cubin));
        unsigned nf = 0;
        CU(cuModuleGetFunctionCount(&nf, mod));
        std::vector<CUfunction> fs(nf);
        CU(cuModuleEnumerateFunctions(fs.data(), nf, mod));
        const CUfunction k_ini = find_kernel(fs, mangled_prefix("procesarAristasDeltaTInicialGPU"));
        const CUfunction k_nocom = find_kernel(fs, mangled_prefix("procesarAristasNoComGPU"));
        const CUfunction k_com = find_kernel(fs, mangled_prefix("procesarAristasComGPU"));
        const CUfunction k_ari = find_kernel(fs, mangled_prefix("procesarAristasGPU"));
        const CUfunction k_dtv = find_kernel(fs, mangled_prefix("obtenerDeltaTVolumenesGPU"));
        const CUfunction k_est = find_kernel(fs, mangled_prefix("obtenerEstadoYDeltaTVolumenesGPU"));
        const CUfunction k_eta = find_kernel(fs, mangled_prefix("actualizarEta1MaximaGPU"));
        if (!k_ini || !k_nocom || !k_com || !k_ari || !k_dtv || !k_est || !k_eta) {
            g_err = "a reference kernel is missing from the cubin";
            return 1;
        }
        // reduce6_min<float, threads>
        auto k_red = [&](int threads) {
            return find_kernel(fs, mangled_prefix("reduce6_min") + "IfLj" + std::to_string(threads) + "E");
        };

        const int N = nx * ny;
        const size_t tex_bytes = size_t(ny + 2) * nx * sizeof(F4), acc_bytes = size_t(N) * sizeof(F4);
        CU(cuMemAlloc(&d_tex1, tex_bytes));
        CU(cuMemAlloc(&d_tex2, tex_bytes));
        CU(cuMemAlloc(&d_acc1, acc_bytes));
        CU(cuMemAlloc(&d_acc2, acc_bytes));
        CU(cuMemAlloc(&d_dtv, size_t(N) * sizeof(float)));
        CU(cuMemAlloc(&d_eta, size_t(N) * sizeof(F2)));
        std::vector<F4> t1(size_t(ny + 2) * nx, F4{0, 0, 0, 0}), t2(t1);
        std::vector<F2> eta(N);
        for (int i = 0; i < N; ++i) {
            t1[nx + i] = F4{state[0][i], state[1][i], state[2][i], state[6][i]};
            t2[nx + i] = F4{state[3][i], state[4][i], state[5][i], state[6][i]};
            eta[i] = F2{state[0][i] + state[3][i] - state[6][i], 0.0f};  // Problema.cxx:542-546
        }
        CU(cuMemcpyHtoD(d_tex1, t1.data(), tex_bytes));
        CU(cuMemcpyHtoD(d_tex2, t2.data(), tex_bytes));
        CU(cuMemcpyHtoD(d_eta, eta.data(), size_t(N) * sizeof(F2)));
        CU(cuMemsetD32(d_acc1, 0, acc_bytes / 4));
        CU(cuMemsetD32(d_acc2, 0, acc_bytes / 4));
        {
            CUdeviceptr sym;
            size_t sz;
            const unsigned long long zero = 0;
            CU(cuModuleGetGlobal(&sym, &sz, mod, "lsh_ref_tex_fault"));
            CU(cuMemcpyHtoD(sym, &zero, sizeof(zero)));
            TexRef tr1{d_tex1, nx, ny + 2}, tr2{d_tex2, nx, ny + 2};
            CU(cuModuleGetGlobal(&sym, &sz, mod, "texDatosVolumenes_1"));
            if (sz != sizeof(TexRef)) { g_err = "texture symbol size"; return 1; }
            CU(cuMemcpyHtoD(sym, &tr1, sizeof(tr1)));
            CU(cuModuleGetGlobal(&sym, &sz, mod, "texDatosVolumenes_2"));
            CU(cuMemcpyHtoD(sym, &tr2, sizeof(tr2)));
        }

        // launch geometry, ShallowWater.cu:34-94 (NUM_HEBRAS_* of Constantes.hxx:81-90)
        const int AA = 8, AL = 8, ACOM = 32, VOL = 256, EA = 8, EL = 8;
        const int ar_ver1 = (nx / 2 + 1) * ny;
        const int ar_ver2 = (nx % 2 == 0) ? nx * ny / 2 : ar_ver1;
        const int ar_hor1 = (ny / 2 + 1) * nx;
        const int ar_hor2 = (ny % 2 == 0) ? nx * ny / 2 : ar_hor1;
        const Launch gV1{k_ari, (unsigned)div_up(ar_ver1 / ny, AA), (unsigned)div_up(ny, AL), AA, AL, 0};
        const Launch gV2{k_ari, (unsigned)div_up(ar_ver2 / ny, AA), (unsigned)div_up(ny, AL), AA, AL, 0};
        const Launch gH1{k_nocom, (unsigned)div_up(nx, AA), (unsigned)div_up(ar_hor1 / nx, AL), AA, AL, 0};
        const Launch gH2{k_ari, (unsigned)div_up(nx, AA), (unsigned)div_up(ar_hor2 / nx, AL), AA, AL, 0};
        const Launch gCom{k_com, (unsigned)div_up(nx, ACOM), 1, ACOM, 2, 0};
        const Launch gEst{k_est, (unsigned)div_up(nx, EA), (unsigned)div_up(ny, EL), EA, EL, 0};
        const Launch gEta{k_eta, (unsigned)div_up(nx, EA), (unsigned)div_up(ny, EL), EA, EL, 0};
        int Nv = N, id_hebra = 0, ultima = 1;
        float dT = 0.0f, t = 0.0f, a1 = angulo1, a2 = angulo2, a3 = angulo3, a4 = angulo4;

        // obtenerMinimoReduccion<float> (Reduccion_kernel.cu:130-172) on d_dtv
        std::vector<float> h_red(4096);
        auto dt_min = [&](float& out) -> int {
            int size = N, blocks = 0, threads = 0;
            if (size > 4096) {
                threads = (size < 256) ? size / 2 : 128;
                blocks = size / (threads * 2);
                if (blocks > 64) blocks = 64;
                CUfunction kr = k_red(threads);
                if (!kr) { g_err = "reduce6_min instantiation missing"; return 1; }
                unsigned un = (unsigned)size;
                void* ra[] = {&d_dtv, &d_dtv, &un};
                CU(cuLaunchKernel(kr, blocks, 1, 1, threads, 1, 1, threads * sizeof(float), nullptr, ra, nullptr));
                // (the reference's second-level loop never runs: blocks <= 64 <= 4096)
                CU(cuMemcpyDtoH(h_red.data(), d_dtv, blocks * sizeof(float)));
                size = blocks;
            } else {
                CU(cuMemcpyDtoH(h_red.data(), d_dtv, size * sizeof(float)));
            }
            out = 1e30f;
            for (int i = 0; i < size; ++i)
                if (h_red[i] < out) out = h_red[i];
            return 0;
        };

        // initial dt (ShallowWater.cu:236-263)
        {
            float bs = borde_sup, bi = borde_inf, bz = borde_izq, bd = borde_der, av = ancho_vol, al = alto_vol;
            float rr = r, g = gravedad, eh = epsilon_h;
            int tipo;
            void* h[] = {&nx, &ny, &Nv, &bs, &bi, &av, &rr, &d_acc1, &g, &eh, &tipo, &id_hebra, &ultima};
            void* v[] = {&nx, &ny, &Nv, &bz, &bd, &al, &rr, &d_acc1, &g, &eh, &tipo, &id_hebra, &ultima};
            Launch i1 = gH1, i2 = gH2, i3 = gV1, i4 = gV2;
            i1.f = i2.f = i3.f = i4.f = k_ini;
            tipo = 3; if (i1.run(h)) return 1;
            tipo = 4; if (i2.run(h)) return 1;
            tipo = 1; if (i3.run(v)) return 1;
            tipo = 2; if (i4.run(v)) return 1;
            float ar = area, cfl = CFL;
            void* d[] = {&d_acc1, &d_dtv, &Nv, &ar, &cfl};
            CU(cuLaunchKernel(k_dtv, div_up(N, VOL), 1, 1, VOL, 1, 1, 0, nullptr, d, nullptr));
            if (dt_min(dT)) return 1;
            CU(cuMemsetD32(d_acc1, 0, acc_bytes / 4));
        }

        std::vector<F4> halo(size_t(nx) * 4, F4{0, 0, 0, 0}), halo_in(size_t(nx) * 4, F4{0, 0, 0, 0});
        const size_t row = size_t(nx) * sizeof(F4);
        auto step = [&]() -> int {
            float tt = t;
            void* ea[] = {&d_eta, &nx, &ny, &tt};
            if (gEta.run(ea)) return 1;
            // halo rows to the host (:362-369)
            CU(cuMemcpyDtoH(&halo[0], d_tex1 + row, row));
            CU(cuMemcpyDtoH(&halo[nx], d_tex2 + row, row));
            CU(cuMemcpyDtoH(&halo[2 * nx], d_tex1 + size_t(ny) * row, row));
            CU(cuMemcpyDtoH(&halo[3 * nx], d_tex2 + size_t(ny) * row, row));
            float bs = borde_sup, bi = borde_inf, bz = borde_izq, bd = borde_der, av = ancho_vol, al = alto_vol;
            float ar = area, rr = r, dt = dT, pe = peso, be = beta, g = gravedad, eh = epsilon_h, LL = L, HH = H;
            int tipo = 3;
            void* h[] = {&nx, &ny, &Nv, &bs, &bi, &av, &ar, &rr, &dt, &a1, &a2, &a3, &a4, &pe, &be,
                         &d_acc1, &d_acc2, &g, &eh, &LL, &HH, &tipo, &id_hebra, &ultima};
            void* v[] = {&nx, &ny, &Nv, &bz, &bd, &al, &ar, &rr, &dt, &a1, &a2, &a3, &a4, &pe, &be,
                         &d_acc1, &d_acc2, &g, &eh, &LL, &HH, &tipo, &id_hebra, &ultima};
            if (gH1.run(h)) return 1;
            // halo rows from the host (:401-408)
            CU(cuMemcpyHtoD(d_tex1, &halo_in[0], row));
            CU(cuMemcpyHtoD(d_tex2, &halo_in[nx], row));
            CU(cuMemcpyHtoD(d_tex1 + size_t(ny + 1) * row, &halo_in[2 * nx], row));
            CU(cuMemcpyHtoD(d_tex2 + size_t(ny + 1) * row, &halo_in[3 * nx], row));
            if (gCom.run(h)) return 1;
            tipo = 4; if (gH2.run(h)) return 1;
            tipo = 1; if (gV1.run(v)) return 1;
            tipo = 2; if (gV2.run(v)) return 1;
            float cfl = CFL, m_c = mfc, m_0 = mf0, m_s = mfs, v1 = vmax1, v2 = vmax2;
            void* es[] = {&d_acc1, &d_acc2, &d_dtv, &nx, &ny, &ar, &cfl, &rr, &dt, &a1, &a2, &a3, &a4,
                          &m_c, &m_0, &m_s, &v1, &v2, &g, &eh, &LL, &HH};
            if (gEst.run(es)) return 1;
            t += dT;
            if (dt_min(dT)) return 1;
            // texture copy-back (:447-450) and accumulator reset (:453-454)
            CU(cuMemcpyDtoD(d_tex1 + row, d_acc1, acc_bytes));
            CU(cuMemcpyDtoD(d_tex2 + row, d_acc2, acc_bytes));
            CU(cuMemsetD32(d_acc1, 0, acc_bytes / 4));
            CU(cuMemsetD32(d_acc2, 0, acc_bytes / 4));
            return 0;
        };
        for (int i = 0; i < warmup; ++i)
            if (step()) return 1;
        CU(cuCtxSynchronize());
        if (dt_trace) dt_trace[0] = dT;
        const auto c0 = std::chrono::steady_clock::now();
        for (int i = 0; i < nsteps; ++i) {
            if (step()) return 1;
            if (dt_trace) dt_trace[i + 1] = dT;
        }
        CU(cuCtxSynchronize());
        const auto c1 = std::chrono::steady_clock::now();
        if (ms_out) *ms_out = std::chrono::duration<double, std::milli>(c1 - c0).count();
        if (t_out) *t_out = t;
        {
            CUdeviceptr sym;
            size_t sz;
            unsigned long long fault = 0;
            CU(cuModuleGetGlobal(&sym, &sz, mod, "lsh_ref_tex_fault"));
            CU(cuMemcpyDtoH(&fault, sym, sizeof(fault)));
            if (fault) {
                g_err = "a reference texture read fell outside its array (x*65536+y+1 = " + std::to_string(fault) + ")";
                return 1;
            }
        }
        CU(cuMemcpyDtoH(t1.data(), d_tex1, tex_bytes));
        CU(cuMemcpyDtoH(t2.data(), d_tex2, tex_bytes));
        for (int i = 0; i < N; ++i) {
            const F4 p1 = t1[nx + i], p2 = t2[nx + i];
            state[0][i] = p1.x; state[1][i] = p1.y; state[2][i] = p1.z;
            state[3][i] = p2.x; state[4][i] = p2.y; state[5][i] = p2.z;
        }
        return 0;
    };
    status = body();
    for (CUdeviceptr p : {d_tex1, d_tex2, d_acc1, d_acc2, d_dtv, d_eta})
        if (p) cuMemFree(p);
    if (mod) cuModuleUnload(mod);
    cuCtxPopCurrent(nullptr);
    cuDevicePrimaryCtxRelease(dev);
    return status;
}

}  // extern "C"
