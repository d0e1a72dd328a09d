/*
 * lsh_compat.h -- drop-in surface for the reference's host code.
 *
 *  - shallowWater(): the reference's solver entry point with its exact
 *    argument list (src/GPU/ShallowWater.cu:125-131, declared in
 *    src/GPU/main.cxx:12-18), running on the GB300 kernels of lsh.h.
 *  - comprobarSoporteCUDA() (src/GPU/ComprobarSoporteCUDA.cu:5).
 *  - lsh_load_datadat(): the data.dat / .bat / .ini loader
 *    (src/GPU/Problema.cxx:139-549), with the reference's istream semantics.
 *  - lsh_nc_*: the six NetCDF-classic output files of src/GPU/netcdf.cu
 *    (<prefix>_eta1.nc ... _q2y.nc), written by this library's own CDF-1 writer.
 *
 * Multi-rank arguments (num_procs, id_hebra, num_voly_otros) are accepted
 * for signature compatibility; only one rank (num_procs == 1, id_hebra == 0)
 * runs -- the GB300 build keeps the whole grid on one GPU.
 */
#ifndef LSH_COMPAT_H
#define LSH_COMPAT_H

#include "lsh.h"

#ifdef __cplusplus
extern "C" {
#endif

/* float4 / float2 with the layout of CUDA's vector types */
typedef struct { float x, y, z, w; } lsh_float4;
typedef struct { float x, y; } lsh_float2;

/* Same memory layout as the reference's TDatoCluster (Constantes.hxx:23-43):
 * datosVolumenes_1[(ny+2)*nx] = (h1, q1x, q1y, H), datosVolumenes_2 = (h2,
 * q2x, q2y, H); row 0 and row ny+1 are halo rows, cell (i, j) is at
 * [(j+1)*nx + i]; eta1_maxima[ny*nx] = (max eta1, time). */
typedef struct lsh_dato_cluster {
    int num_volx, num_voly;
    lsh_float4* datosVolumenes_1;
    lsh_float4* datosVolumenes_2;
    lsh_float2* eta1_maxima;
    lsh_float4* puntero_datosVolumenesComClusterSup_1;
    lsh_float4* puntero_datosVolumenesComClusterSup_2;
    lsh_float4* puntero_datosVolumenesComClusterInf_1;
    lsh_float4* puntero_datosVolumenesComClusterInf_2;
    lsh_float4* puntero_datosVolumenesComOtroClusterSup_1;
    lsh_float4* puntero_datosVolumenesComOtroClusterSup_2;
    lsh_float4* puntero_datosVolumenesComOtroClusterInf_1;
    lsh_float4* puntero_datosVolumenesComOtroClusterInf_2;
} lsh_dato_cluster;

/* shallowWater (ShallowWater.cu:125-486): runs the time loop to tiempo_tot
 * (t < tiempo_tot, :269) with the reference's first-order scheme in FP64 on
 * the GPU, writes NetCDF snapshots every tiempo_guardar (>= 0) or, when
 * leer_fichero_puntos == 1, the gauge text file <prefijo>_eta_puntos.txt,
 * and leaves the final state and eta1 max in datos_cluster (float).  Returns
 * 0 ok, 1 not enough GPU memory, 2 not enough CPU memory (as the reference),
 * 3 other errors.  *tiempo receives the loop's wall time in seconds. */
int shallowWater(lsh_dato_cluster* datos_cluster, float xmin, float ymin, float Hmin, char* nombre_bati,
                 char* prefijo, int num_voly_otros, int num_voly_total, float borde_sup, float borde_inf,
                 float borde_izq, float borde_der, float ancho_vol, float alto_vol, float area, float tiempo_tot,
                 float tiempo_guardar, float CFL, float r, float angulo1, float angulo2, float angulo3,
                 float angulo4, float peso, float beta, float mfc, float mf0, float mfs, float vmax1, float vmax2,
                 float gravedad, float epsilon_h, float L, float H, float Q, float T, int num_procs, int id_hebra,
                 double* tiempo, int leer_fichero_puntos, int* indiceVolumenesGuardado,
                 int* posicionesVolumenesGuardado, int num_puntos_guardar);

/* comprobarSoporteCUDA (ComprobarSoporteCUDA.cu:5-25): 0 ok, 1 no GPU,
 * 2 no CUDA-capable GPU. */
int comprobarSoporteCUDA(void);

/* A problem read from data.dat (cargarDatosProblema, Problema.cxx:139-549),
 * normalised as the reference does (L, H -> Q, T, g = 1 when normalizar == 1)
 * and with the depth shift H -= Hmin when land exists (:463-481).  State
 * arrays are FP64, row-major nx*ny (row 0 = the first row of the .bat/.ini
 * files).  The loader owns every pointer; free with lsh_problem_free. */
typedef struct lsh_problem {
    lsh_params params;          /* nx, ny, dx, dy, borders, CFL, r, angle1..4, mfc, mf0, mfs, vmax, g, eps_h, L, H */
    double xmin, xmax, ymin, ymax;
    double hmin;                /* Hmin_global (<= 0), already subtracted from H */
    double Q, T;                /* normalisation scales */
    double tiempo_tot, tiempo_guardar;
    int32_t leer_fichero_puntos;
    int32_t num_puntos_guardar;
    int32_t* indice_puntos;     /* [num_puntos_guardar] cell index or -1 */
    double* state[LSH_NVARS];   /* h1 q1x q1y h2 q2x q2y H */
    double* eta1_max;           /* initial eta1 max = h1 + h2 - H (Problema.cxx:542-546) */
    char nombre_bati[256];
    char prefijo[512];
    char error[512];            /* message when loading failed */
} lsh_problem;

/* Returns LSH_OK, LSH_ERR_IO (missing / malformed file; see p->error) or
 * LSH_ERR_HOST_OOM.  On failure *out may still hold the error text. */
int lsh_load_datadat(const char* path, lsh_problem** out);
/* Same, choosing the friction law the data file is written for: Pouliquen
 * files carry four angles (the reference's #ifndef COULOMB build). */
int lsh_load_datadat_law(const char* path, int friction_law, lsh_problem** out);
void lsh_problem_free(lsh_problem* p);

/* The six NetCDF-classic files of netcdf.cu (initNC / writerecs / closeNC).
 * Values are passed already in output units (metres, m^2/s, seconds).
 * bathymetry and x / y cell-centre axes are written at creation. */
typedef struct lsh_nc lsh_nc;
int lsh_nc_create(const char* prefix, const char* nombre_bati, int nx, int ny, const float* x, const float* y,
                  const float* bathymetry, float tiempo_tot, float CFL, float r, const float angles_deg[4],
                  int pouliquen, float mfc, float mf0, float mfs, float vmax1, float vmax2, lsh_nc** out);
/* one record: time and the six fields (nx*ny each) */
int lsh_nc_write(lsh_nc* nc, float time, const float* eta1, const float* q1x, const float* q1y,
                 const float* eta2, const float* q2x, const float* q2y);
/* writes max_height (nx*ny, may be NULL) and closes all files */
int lsh_nc_close(lsh_nc* nc, const float* max_height);

#ifdef __cplusplus
}
#endif
#endif /* LSH_COMPAT_H */
