/*
 * cholla_oracle.h -- FP64 CPU restatement of Cholla's single-GPU VL hydro/MHD step.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity checker and the CPU
 * baseline.  Nothing in the cholla_gb300 product links, loads or calls it; only
 * tests/, __graft_entry__.smoke() and bench.py (cpu_baseline / --impl reference)
 * may use it.
 *
 * Each function restates one kernel of the reference (cholla-hydro/cholla) over
 * the full padded grid, in the reference's operation order, so that this code
 * compiled with -ffp-contract=off reproduces the reference's -fmad=false build.
 * The file:line of the reference kernel each function follows is given beside it.
 *
 * Layout (src/grid/grid_enum.h:18-111): field-major U[f*n_cells + i + j*nx + k*nx*ny],
 * fields d, mx, my, mz, E, [scalars], [Bx, By, Bz], [GasEnergy (last)].
 */
#pragma once
#include <cstddef>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_PCM = 0, ORC_PLMC = 1, ORC_PPMC = 2, ORC_PLMP = 3, ORC_PPMP = 4 };
enum { ORC_HLLC = 0, ORC_ROE = 1, ORC_HLLD = 2, ORC_HLL = 3, ORC_EXACT = 4 };

typedef struct {
  int nx, ny, nz;     /* padded sizes (ghosts included) */
  int n_ghost;
  int n_fields;
  int n_scalars;
  int de;             /* dual energy on */
  int mhd;            /* MHD (face-centred B, CT) */
  int recon;          /* ORC_PCM / ORC_PLMC / ORC_PPMC / ORC_PLMP / ORC_PPMP */
  int solver;         /* ORC_HLLC / ORC_ROE / ORC_HLLD / ORC_HLL / ORC_EXACT */
  int density_floor_on;
  double gamma;
  double dx, dy, dz;
  double density_floor;
} orc_config;

/* ---- kernel-level restatements (write into caller-owned full-grid arrays) ---- */
void orc_pcm_3d(const orc_config *c, const double *U, double *QLx, double *QRx, double *QLy, double *QRy,
                double *QLz, double *QRz);
void orc_ppmc_vl(const orc_config *c, const double *U, double *QL, double *QR, int dir);
void orc_plmc(const orc_config *c, const double *U, double *QL, double *QR, int dir);
/* primitive-limited PLM / PPM (plmp_cuda.cu:21-365, ppmp_cuda.cu:28-752; hydro only) */
void orc_plmp(const orc_config *c, const double *U, double *QL, double *QR, int dir);
void orc_ppmp(const orc_config *c, const double *U, double *QL, double *QR, int dir);
void orc_hllc(const orc_config *c, const double *QL, const double *QR, double *F, int dir);
void orc_roe(const orc_config *c, const double *QL, const double *QR, double *F, int dir);
void orc_hlld(const orc_config *c, const double *QL, const double *QR, const double *Bface, double *F, int dir);
/* hll_cuda.cu:19-268 and exact_cuda.cu:19-334 (hydro; the exact solver's fractional powers in
 * single precision, as the reference's powf) */
void orc_hll(const orc_config *c, const double *QL, const double *QR, double *F, int dir);
void orc_exact(const orc_config *c, const double *QL, const double *QR, double *F, int dir);
/* one CT slope at cell (x, y, z) (ct_electric_fields.h:66-120 _ctSlope) */
double orc_ct_slope(const orc_config *c, const double *flux, const double *U, double flux_sign, int ct_dir, int cq1,
                    int cq2, int fq1, int fq2, int x, int y, int z);
void orc_ct_electric_fields(const orc_config *c, const double *Fx, const double *Fy, const double *Fz,
                            const double *U, double *emf);
void orc_update_magnetic(const orc_config *c, const double *src, double *dst, const double *emf, double dt);
void orc_update_half(const orc_config *c, const double *U, double *Uh, const double *Fx, const double *Fy,
                     const double *Fz, double dt_half);
void orc_de_partial_update(const orc_config *c, double *U, double dt);
void orc_update_full(const orc_config *c, double *U, const double *Fx, const double *Fy, const double *Fz,
                     double dt);
void orc_de_select(const orc_config *c, double *U);
void orc_de_sync(const orc_config *c, double *U);
void orc_temperature_floor(const orc_config *c, double *U, double U_floor);
double orc_calc_dt(const orc_config *c, const double *U);
/* max |div B| over the cells with x, y, z >= 2 of the whole box, ghost layers included */
double orc_max_divB(const orc_config *c, const double *U);
void orc_set_boundaries(const orc_config *c, double *U, const int flags[6]);

/* PPM single-variable reconstruction (reconstruction.h:794-901) */
void orc_ppm_single_variable(double im2, double im1, double i, double ip1, double ip2, double *L_iph,
                             double *R_imh);

/* ---- reconstruction building blocks, for the reference's helper unit tests
 * (src/reconstruction/reconstruction_tests.cu).  Primitive states are 9 doubles (density,
 * vx, vy, vz, pressure, Bx, By, Bz, gas energy), characteristic states 7, MHD eigenvector sets
 * the 18 members of reconstruction::EigenVecs in order.  dir 0/1/2 picks the x/y/z
 * permutation of the momenta. ---- */
int orc_t_thread_guard(const orc_config *c, int order, int x, int y, int z);                          /* :95-119 */
void orc_t_load_data(const orc_config *c, const double *U, int x, int y, int z, int dir, double *out); /* :139-212 */
void orc_t_write_data(const orc_config *c, const double *state, double *Q, const double *U, size_t id,
                      int dir);                                                                        /* :918-968 */
void orc_t_compute_slope(const orc_config *c, const double *left, const double *right, double coef,
                         double *out);                                                                 /* :224-247 */
void orc_t_van_leer_slope(const orc_config *c, const double *left, const double *right, double *out); /* :258-296 */
void orc_t_eigenvectors(const double *prim, double cs, double cs2, double gamma, double *out);        /* :310-361 */
void orc_t_prim_to_char(int mhd, const double *prim, const double *slope, const double *eig, double cs, double cs2,
                        double *out);                                                                  /* :378-437 */
void orc_t_char_to_prim(int mhd, const double *prim, const double *chr, const double *eig, double cs, double cs2,
                        double *out);                                                                  /* :453-491 */
/* del = {del_L, del_R, del_C, del_G} (primitive), del_a = the same four in characteristic variables */
void orc_t_monotonize_characteristic(const orc_config *c, const double *prim, const double *const del[4],
                                     const double *const del_a[4], const double *eig, double cs, double cs2,
                                     double *out);                                                     /* :512-559 */
void orc_t_calc_interface_linear(const orc_config *c, const double *cell, const double *slope, double sign,
                                 double *out);                                                         /* :645-673 */
void orc_t_plm_limit_interfaces(const orc_config *c, double *l_iph, double *r_imh, const double *cell_im1,
                                const double *cell_i, const double *cell_ip1);                         /* :686-723 */

/* ---- hydro / MHD utilities on the path (hydro_utilities.h, mhd_utilities.h), for the reference's
 * utility unit tests (src/utils/hydro_utilities_tests.cpp, mhd_utilities_tests.cu) ---- */
double orc_t_pressure_primitive(double E, double d, double vx, double vy, double vz, double gamma, int mhd, double bx,
                                double by, double bz);
double orc_t_energy_primitive(double P, double d, double vx, double vy, double vz, double gamma, int mhd, double bx,
                              double by, double bz);
double orc_t_pressure_from_de(double E, double U_total, double U_advected, double gamma);
double orc_t_kinetic_energy(double d, double vx, double vy, double vz);
double orc_t_magnetic_energy(double bx, double by, double bz);
double orc_t_total_pressure(double p, double bx, double by, double bz);
double orc_t_fast_magnetosonic(double d, double p, double bx, double by, double bz, double gamma);
double orc_t_slow_magnetosonic(double d, double p, double bx, double by, double bz, double gamma);
double orc_t_alfven_speed(double bx, double d);
/* the three cell-centred fields of cell (x, y, z) at flat index id of a grid with the given
 * x / y strides and n_cells per field, magnetic_x at field fB */
void orc_t_cell_centered_b(const double *U, size_t id, int x, int y, int z, size_t n_cells, int nx, int ny, int fB,
                           double *out);

/* ---- HLLD building blocks, for the reference's HLLD-internal unit tests
 * (src/riemann_solvers/hlld_cuda_tests.cu:1877-2400).  Packed in the member order of
 * mhd::internal::State (9 doubles), StarState (6), DoubleStarState (6), Flux (7), Speeds (5). ---- */
void orc_t_hlld_load_state(const orc_config *c, const double *Q, double bx, size_t t, int dir, double *out);
void orc_t_hlld_return_fluxes(const orc_config *c, size_t t, int dir, double *F, const double *flux,
                              const double *state);
void orc_t_hlld_lr_speeds(const double *stateL, const double *stateR, double bx, double gamma, double *speeds);
double orc_t_hlld_middle_speed(const double *stateL, const double *stateR, const double *speeds);
double orc_t_hlld_star_speed(const double *star, const double *speeds, double bx, double side);
double orc_t_hlld_star_total_pressure(const double *stateL, const double *stateR, const double *speeds);
void orc_t_hlld_nonstar_fluxes(const double *state, double bx, double *flux);
void orc_t_hlld_star_state(const double *state, const double *speeds, double S, double bx, double pt_star,
                           double *star);
void orc_t_hlld_star_fluxes(const double *star, const double *state, const double *flux, const double *speeds,
                            double S, double *out);
void orc_t_hlld_double_star_state(const double *starL, const double *starR, double bx, double pt_star,
                                  const double *speeds, double *out);
void orc_t_hlld_double_star_fluxes(const double *dstar, double dstar_energy, const double *star, const double *state,
                                   const double *flux, const double *speeds, double S, double S_star, double *out);

/* ---- the step: VL_Algorithm_3D_CUDA / VL_Algorithm_1D_CUDA ---- */
int orc_vl_step_3d(const orc_config *c, double *U, double dt);
int orc_vl_step_1d(const orc_config *c, double *U, double dt);
/* src/integrators/VL_2D_cuda.cu:25-174 VL_Algorithm_2D_CUDA (nz = 1; hydro; no HLL or HLLD) */
int orc_vl_step_2d(const orc_config *c, double *U, double dt);

/* std::mt19937_64(seed) + std::uniform_real_distribution<double>(a, b), n draws: the input
 * generator of the reference's unit tests (e.g. src/reconstruction/ppmc_cuda_tests.cu:131-132) */
void orc_mt19937_uniform(unsigned long long seed, double a, double b, size_t n, double *out);
/* the same with the 32-bit std::mt19937 (src/mhd/magnetic_divergence_tests.cu:47-48,
 * src/mhd/ct_electric_fields_tests.cu:197-198) */
void orc_mt19937_32_uniform(unsigned long seed, double a, double b, size_t n, double *out);

/* threads used by the OpenMP loops (0 = library default) */
void orc_set_threads(int n);
int orc_get_threads(void);

#ifdef __cplusplus
}
#endif
