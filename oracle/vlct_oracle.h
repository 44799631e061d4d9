/*
 * vlct_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of Enzo-E's VL+CT MHD step (Method "mhd_vlct"), used as the
 * parity oracle for the CUDA implementation.  Nothing in the product links or
 * calls this code: only tests/, __graft_entry__.smoke() and bench.py's
 * cpu_baseline leg load it, and only as the checker / CPU baseline.
 *
 * Block layout is Cello's (src/Cello/data_FieldData.cpp:585-619): row-major
 * (z, y, x), x fastest.  Cell fields are (mz, my, mx) with m = n + 2g; the
 * face field bfieldi_d has one extra entry along axis d.
 */
#ifndef VLCT_ORACLE_H
#define VLCT_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_HLLE = 0, ORC_HLLC = 1, ORC_HLLD = 2 };
enum { ORC_NN = 0, ORC_PLM = 1, ORC_PLM_ATHENA = 2 };

typedef struct {
  int riemann;          /* ORC_HLLE / ORC_HLLC / ORC_HLLD                     */
  int recon;            /* reconstruction of the full-dt (last) stage         */
  int mhd;              /* 1: constrained_transport, 0: no_bfield             */
  int dual_energy;      /* 1: "modern" dual-energy formalism                  */
  int euler;            /* 1: time_scheme "euler" (one stage), 0: "vl"        */
  double eta;           /* dual-energy eta                                    */
  double theta_limiter;
  double gamma;
  double density_floor;
  double pressure_floor;
  double courant;
} OracleParams;

typedef struct {
  int nx, ny, nz;       /* active cells per axis                              */
  int g;                /* ghost depth (same on every axis)                   */
  double dx, dy, dz;    /* cell widths                                        */
  double *rho, *vx, *vy, *vz, *etot, *eint;      /* eint may be NULL          */
  double *bx, *by, *bz;                          /* cell-centred B (MHD)      */
  double *bfx, *bfy, *bfz;                       /* face-centred B (MHD)      */
  double *pressure;                              /* [w] scratch field         */
  double *ax, *ay, *az;  /* acceleration_x/y/z (gravity source), or NULL     */
  double *passive[4];    /* passively advected scalars, conserved form (a     */
  int npassive;          /* density), npassive <= 4                           */
} OracleBlock;

/* The step with store_fluxes_for_corrections (hydro only): after the final
 * stage, out[(dim * 2 + side) * nq + iq] receives dt/dx_dim times the flux of
 * quantity quantities[iq] (0 density, 1-3 velocity x/y/z, 4 total energy,
 * 5 internal energy) through the low (side 0) or high (side 1) active face of
 * axis dim, as arrays (nz, ny) / (nz, nx) / (ny, nx), last index fastest
 * (EnzoMethodMHDVlct.cpp:250-330).  Returns 4 with magnetic fields. */
int oracle_step_fc(const OracleParams* p, OracleBlock* b, double dt,
                   double* const* out, int nq, const int* quantities);

/* One full VL+CT step of size dt on one ghosted block, in place.  Returns 0,
 * or 3 for the euler scheme with magnetic fields (the reference ERRORs:
 * EnzoBfieldMethod.cpp:23-27). */
int oracle_step(const OracleParams* p, OracleBlock* b, double dt);

/* The Method::timestep of the reference: syncs energies (dual energy), writes
 * the pressure field over the whole ghosted block and returns
 * courant * min_cells min_d dx_d / (|v_d| + c_fast).                        */
double oracle_timestep(const OracleParams* p, OracleBlock* b);

/* Same-level periodic ghost refresh of one block onto itself (Cello rules). */
void oracle_fill_ghosts_periodic(OracleBlock* b);

/* Refresh of a set of equal-sized blocks on a periodic nbx x nby x nbz brick.
 * blocks[(kz*nby + ky)*nbx + kx]. */
void oracle_fill_ghosts_brick(OracleBlock* blocks, int nbx, int nby, int nbz);

/* Enzo-E's inclined linear-wave initial condition (EnzoInitialInclinedWave)
 * for wave in {"fast","alfven","slow","mhd_entropy","sound","hd_entropy"},
 * on a single block whose lower domain corner is (x0,y0,z0). */
int oracle_ic_inclined_wave(OracleBlock* b, const char* wave, double alpha,
                            double beta, double gamma, double amplitude,
                            double lambda, int positive_vel, double x0,
                            double y0, double z0);

/* Cello-style driver for one periodic block: repeated timestep / refresh /
 * step until stop_time.  Returns the number of cycles taken. */
int oracle_evolve_periodic(const OracleParams* p, OracleBlock* b,
                           double stop_time, int max_cycles);

/* Number of floating-point operations of the last oracle_step (when built
 * with op counting), else -1. */
long long oracle_flop_count(void);

#ifdef __cplusplus
}
#endif
#endif
