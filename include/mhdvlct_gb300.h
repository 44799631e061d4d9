/*
 * mhdvlct_gb300.h -- C ABI of the GB300 VL+CT magnetohydrodynamics step.
 *
 * Drop-in for Enzo-E's Method "mhd_vlct" (src/Enzo/hydro-mhd/
 * EnzoMethodMHDVlct.{hpp,cpp}).  The Cello plugin boundary is the Method
 * interface (src/Cello/problem_Method.hpp:23-124): compute(Block*) and
 * timestep(Block*).  This header exposes the same two operations on one
 * ghosted block held in device memory in Cello's layout, plus the ghost
 * refresh that Cello performs between them, a batched form over many blocks
 * and a serving loop over independent solves.
 *
 * Conventions
 *  - Every function returns 0 on success and a positive MHD_ERR_* code on
 *    failure; none aborts.  mhdvlct_last_error_string() describes the last
 *    failure of a handle.
 *  - Field arrays follow Cello's FieldData layout
 *    (src/Cello/data_FieldData.cpp:585-619): row-major (z, y, x), x fastest,
 *    extent n + 2g per axis, no padding; the face-centred field bfieldi_d has
 *    one extra entry along axis d.
 *  - Block-level device memory is caller-owned; batch and serving memory is
 *    library-owned.  One handle per host thread.
 *  - `stream` is a cudaStream_t passed as void* (NULL = legacy stream).
 */
#ifndef MHDVLCT_GB300_H
#define MHDVLCT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- errors */
enum {
  MHD_OK = 0,
  MHD_ERR_INVALID = 1,     /* bad argument or unsupported combination      */
  MHD_ERR_CUDA = 2,        /* a CUDA call failed                           */
  MHD_ERR_NOMEM = 3,       /* device allocation failed / over budget       */
  MHD_ERR_GHOST = 4,       /* ghost depth too small for the stages         */
  MHD_ERR_NONFINITE = 5,   /* a non-finite value was detected              */
  MHD_ERR_TIMEOUT = 6,     /* a bounded wait ran out                       */
  MHD_ERR_BUSY = 7         /* request not finished / queue full            */
};

enum { MHD_DTYPE_F64 = 0, MHD_DTYPE_F32 = 1 };

/* -------------------------------------------------------------- params
 * The Method:mhd_vlct parameter block and the fluid properties it uses
 * (EnzoMethodMHDVlct.cpp:39-101; Physics:fluid_props in
 * src/Enzo/enzo-core/EnzoConfig.cpp:952-1262).  Defaults as in the
 * reference: riemann_solver "hlld", time_scheme "vl", reconstruct_method
 * "plm", theta_limiter 1.5, courant 0.3 (vl), gamma 5/3, dual-energy eta
 * 0.001.  mhd_choice has no default (the reference ERRORs when it is unset). */
typedef struct MhdVlctParams {
  char mhd_choice[32];          /* "constrained_transport" | "no_bfield"      */
  char riemann_solver[16];      /* "hlle" | "hllc" | "hlld"                   */
  char time_scheme[16];         /* "vl" | "euler"                             */
  char reconstruct_method[16];  /* "nn" | "plm" | "plm_enzo" | "plm_athena"   */
  double theta_limiter;
  double courant;
  double gamma;
  double density_floor;
  double pressure_floor;
  int dual_energy;              /* 0: disabled, 1: "modern" formulation       */
  double dual_energy_eta;
} MhdVlctParams;

/* Fill with the reference defaults (mhd_choice left empty). */
void mhdvlct_params_default(MhdVlctParams* p);

/* Parse a Cello-style parameter text such as
 *   Method { mhd_vlct { mhd_choice = "constrained_transport";
 *                       riemann_solver = "hlld"; courant = 0.4; }; }
 *   Physics { fluid_props { eos { gamma = 1.6666666666666667; }
 *             floors { density = 1e-200; pressure = 1e-200; }
 *             dual_energy { type = "modern"; eta = 0.001; } } }
 * Only the keys of this path are read; others are ignored.  Returns
 * MHD_ERR_INVALID with a message in errbuf on a malformed value. */
int mhdvlct_params_parse(const char* text, MhdVlctParams* out, char* errbuf,
                         size_t errbuf_len);

/* --------------------------------------------------------------- handle */
typedef struct mhdvlct_handle mhdvlct_handle;

/* EnzoMethodMHDVlct::EnzoMethodMHDVlct (EnzoMethodMHDVlct.cpp:90-152):
 * validates the parameters (HLLC requires no_bfield, HLLE/HLLD require
 * constrained_transport, theta in [1, 2], ...). */
int mhdvlct_create(const MhdVlctParams* params, mhdvlct_handle** out);
int mhdvlct_destroy(mhdvlct_handle* h);
const char* mhdvlct_last_error_string(const mhdvlct_handle* h);
/* Courant factor in effect (the "courant" key, default 0.3 for "vl" and 1 for
 * "euler", EnzoMethodMHDVlct.cpp:100-101). */
double mhdvlct_courant(const mhdvlct_handle* h);
/* Sum of ghost depths the stages consume (NN + PLM = 3), the minimum ghost
 * depth a block must have (EnzoMethodMHDVlct.cpp:124-133). */
int mhdvlct_required_ghost_depth(const mhdvlct_handle* h);

/* ------------------------------------------------------------ one block */
typedef struct MhdBlockView {
  int dtype;              /* MHD_DTYPE_F64 or MHD_DTYPE_F32                  */
  int n[3];               /* active cells along x, y, z                      */
  int ghost[3];           /* ghost depth along x, y, z (must be equal)       */
  double cell_width[3];   /* EnzoBlock::CellWidth                            */
  void* density;
  void* velocity[3];      /* velocity_x/y/z (specific)                       */
  void* total_energy;     /* specific total energy                           */
  void* internal_energy;  /* specific internal energy (dual energy only)     */
  void* bfield[3];        /* cell-centred bfield_x/y/z (MHD only)            */
  void* bfieldi[3];       /* face-centred bfieldi_x/y/z (MHD only)           */
  void* pressure;         /* [w] pressure field; may be NULL                 */
  void* acceleration[3];  /* acceleration_x/y/z for the gravity source term
                           * (EnzoSourceGravity.cpp:17-69, applied on the
                           * full-dt stage of the vl scheme); all three or
                           * none (NULL)                                      */
  void* passive[4];       /* passively advected scalars in conserved form (a
                           * density), e.g. Cello's "colour" fields
                           * (EnzoIntegrationQuanUpdate.cpp:242-270)         */
  int npassive;           /* number of passive scalars, 0..4                 */
} MhdBlockView;

/* EnzoMethodMHDVlct::compute (EnzoMethodMHDVlct.cpp:356-500): one VL+CT step
 * of size dt on a block whose ghost zones have been refreshed, in place. */
int mhdvlct_block_step(mhdvlct_handle* h, const MhdBlockView* b, double dt,
                       void* stream);

/* Flux correction (store_fluxes_for_corrections, EnzoMethodMHDVlct.cpp:
 * 136-141, 250-330, 483-490): the step additionally writes dt/dx_axis times
 * the flux of selected integration quantities through the low (side 0, face
 * between cells g-1 and g) and high (side 1, face between cells g+n-1 and
 * g+n) active boundary of every axis, as Cello's FluxData holds them.
 * flux[axis][side][quantity] is a device array of the block's active face in
 * the block's dtype, last index fastest: axis 0 (nz, ny), axis 1 (nz, nx),
 * axis 2 (ny, nx); NULL entries are skipped.  Hydro only (the reference
 * asserts it); internal_energy needs dual energy.  The passive scalars'
 * fluxes (their conserved-form flux: the density flux times the upwind
 * specific scalar) are stored like any other field of the flux-correction
 * group, as the reference's FluxData holds every field of its "conserved"
 * group (EnzoMethodMHDVlct.cpp:265-272): MHD_Q_PASSIVE_0 + k needs
 * npassive > k. */
enum {
  MHD_Q_DENSITY = 0,
  MHD_Q_VELOCITY_X = 1, /* the x-momentum flux, as the reference keys it */
  MHD_Q_VELOCITY_Y = 2,
  MHD_Q_VELOCITY_Z = 3,
  MHD_Q_TOTAL_ENERGY = 4,
  MHD_Q_INTERNAL_ENERGY = 5,
  MHD_Q_PASSIVE_0 = 6,  /* .. MHD_Q_PASSIVE_0 + 3: MhdBlockView::passive[k] */
  MHD_FC_NQ = 10
};
typedef struct MhdFluxCorrection {
  void* flux[3][2][MHD_FC_NQ];
} MhdFluxCorrection;
int mhdvlct_block_step_fc(mhdvlct_handle* h, const MhdBlockView* b, double dt,
                          const MhdFluxCorrection* fc, void* stream);

/* EnzoMethodMHDVlct::timestep (EnzoMethodMHDVlct.cpp:551-588): energy sync
 * (dual energy), pressure field, courant * CFL dt over the whole ghosted
 * block.  Synchronises `stream` to return dt on the host. */
int mhdvlct_block_timestep(mhdvlct_handle* h, const MhdBlockView* b,
                           double* dt_out, void* stream);

/* The timestep, the dt reduction and the step with dt kept on the device, so
 * that a process driving many blocks through the per-block calls never waits
 * for the GPU inside a cycle: each block's dt goes to a device slot
 * (EnzoMethodMHDVlct::timestep, EnzoMethodMHDVlct.cpp:551-588), one call
 * takes the minimum over the slots (Cello's min-reduction over blocks,
 * src/Cello/control_stopping.cpp:96-106), and every block's step reads that
 * minimum on the device (EnzoMethodMHDVlct::compute with block->dt(),
 * EnzoMethodMHDVlct.cpp:356-500).  All three only enqueue work on `stream`;
 * dt_dev / dt_min_dev are device pointers to doubles owned by the caller.
 * The step does not check the dt it reads: it must be positive and finite
 * when the step runs. */
int mhdvlct_block_timestep_device(mhdvlct_handle* h, const MhdBlockView* b,
                                  double* dt_dev, void* stream);
int mhdvlct_dt_min_device(mhdvlct_handle* h, const double* dt_dev, int n,
                          double* dt_min_dev, void* stream);
int mhdvlct_block_step_device_dt(mhdvlct_handle* h, const MhdBlockView* b,
                                 const double* dt_dev, void* stream);

/* No counterpart in the reference (the reference's compute allocates its
 * scratch through EnzoVlctScratchSpace on the host heap).  For callers that
 * cannot call cudaMalloc: a host whose device memory is all claimed up front
 * by its own allocator (a pool sized at start-up), or one that must not make
 * a call that may synchronise the whole device while other streams run.
 * Same operation and results as mhdvlct_block_step, but allocates no device
 * memory: its scratch
 * is one file-scope __device__ array of 8 MiB (8388608 bytes) per device,
 * whose address is taken with cudaGetSymbolAddress on the first call on each
 * device and cached.  Make that first call on a device outside stream
 * capture.  A block whose scratch (all cell fields, the passive scalars'
 * half step and two sets of face fields at the ghosted extents, plus
 * descriptors) exceeds 8 MiB, or whose
 * stage needs more than 1024 tiles, is rejected with MHD_ERR_INVALID and a
 * message naming the bytes needed (an FP64 block of 32^3 cells with 3 ghost
 * zones needs about 6.7 MB).  Nothing in the array has to start at zero:
 * every call rewrites the dt slot, the stage descriptors and the tile list,
 * and each intermediate value a stage reads was written earlier in the same
 * call.  All calls on one device share the array: two calls that overlap in
 * time (different streams, threads or handles) race on it; order them on one
 * stream or synchronise between them. */
int mhdvlct_block_step_noalloc(mhdvlct_handle* h, const MhdBlockView* b,
                               double dt, void* stream);

/* Initial face-centred B as the curl of an edge-centred vector potential,
 * then the centred B (EnzoInitialBCenter::initialize_bfield_interface and
 * ::initialize_bfield_center, src/Enzo/initial/EnzoInitialBCenter.cpp:27-127):
 * computed in double and cast to the block's type.  ax, ay, az are device
 * arrays in double with extents (x, y, z) = (m0, m1+1, m2+1), (m0+1, m1,
 * m2+1), (m0+1, m1+1, m2) for the ghosted extents m, x fastest. */
int mhdvlct_block_bfield_from_potential(mhdvlct_handle* h, const MhdBlockView* b,
                                        const double* ax, const double* ay,
                                        const double* az, void* stream);

/* Same-level periodic ghost refresh of a block onto itself (the effect of
 * Cello's refresh for a single periodic root block,
 * src/Cello/control_refresh.cpp:243-360). */
int mhdvlct_fill_ghosts_periodic(mhdvlct_handle* h, const MhdBlockView* b,
                                 void* stream);

/* ------------------------------------------------- mesh ghost refresh
 * Cello's ghost refresh between the leaf blocks of a mesh whose neighbours
 * may sit one level coarser or finer (Block::refresh_load_field_faces_ and
 * refresh_load_field_face_, src/Cello/control_refresh.cpp:243-360; the
 * per-face work of FieldFace::face_to_face, src/Cello/data_FieldFace.cpp:
 * 440-566) with the "linear" operators: restriction (RestrictLinear,
 * src/Cello/problem_RestrictLinear.cpp:53-196) into a coarser receiver and
 * prolongation (ProlongLinear, src/Cello/problem_ProlongLinear.cpp:79-310)
 * into a finer one.  One face is one (sender, receiver) pair as Cello's
 * neighbour iterator yields it, described from the sender's side. */
enum { MHD_REFRESH_COARSE = -1, MHD_REFRESH_SAME = 0, MHD_REFRESH_FINE = 1 };

typedef struct MhdRefreshFace {
  int sender;    /* index of the sending block in the blocks[] array        */
  int receiver;  /* index of the receiving block                             */
  int type;      /* the receiver's level relative to the sender's:
                  * MHD_REFRESH_COARSE (restrict), _SAME (copy), _FINE
                  * (prolong)                                                */
  int face[3];   /* the sender's face toward the receiver, -1/0/+1 per axis  */
  int child[3];  /* _COARSE: the sender's child index within its parent;
                  * _FINE: the receiver's child index within its parent;
                  * _SAME: ignored (0/1 per axis)                            */
} MhdRefreshFace;

/* Field slots, as used by the `conservative` mask below. */
enum {
  MHD_FIELD_DENSITY = 0,
  MHD_FIELD_VELOCITY_X = 1, MHD_FIELD_VELOCITY_Y = 2, MHD_FIELD_VELOCITY_Z = 3,
  MHD_FIELD_TOTAL_ENERGY = 4,
  MHD_FIELD_INTERNAL_ENERGY = 5,
  MHD_FIELD_BFIELD_X = 6, MHD_FIELD_BFIELD_Y = 7, MHD_FIELD_BFIELD_Z = 8,
  MHD_FIELD_PRESSURE = 9,
  MHD_FIELD_ACCELERATION_X = 10, MHD_FIELD_ACCELERATION_Y = 11,
  MHD_FIELD_ACCELERATION_Z = 12,
  MHD_FIELD_PASSIVE_0 = 13, /* .. MHD_FIELD_PASSIVE_0 + 3 */
  MHD_FIELD_BFIELDI_X = 17, MHD_FIELD_BFIELDI_Y = 18, MHD_FIELD_BFIELDI_Z = 19,
  MHD_NFIELD_SLOTS = 20
};
/* The "make_field_conservative" group of the reference's flux-correction
 * decks (input/FluxCorrect/inclined_contact.incl): velocities and total
 * energy are interpolated as density-weighted quantities across levels. */
#define MHD_CONSERVATIVE_DEFAULT                                               \
  ((1u << MHD_FIELD_VELOCITY_X) | (1u << MHD_FIELD_VELOCITY_Y) |               \
   (1u << MHD_FIELD_VELOCITY_Z) | (1u << MHD_FIELD_TOTAL_ENERGY))

/* Refresh the ghost zones named by `faces` in one launch.  Every block has the
 * same active size, ghost depth and dtype (as in Cello); every field present
 * (non-NULL) in the views is refreshed, density first.  Cell fields in the
 * `conservative` mask (bit MHD_FIELD_*) are multiplied by the sender's
 * density before a restriction or prolongation and divided by the receiver's
 * refreshed density after it (FieldFace::mul_by_density_ / div_by_density_,
 * data_FieldFace.cpp:863-980); the sender's own values are left untouched.
 * Face-centred B is refreshed between same-level blocks only: the reference
 * has no restriction or prolongation for it (its ProlongLinear rejects the
 * face-centred extents).  Returns MHD_ERR_INVALID where the reference would
 * assert: a prolongation whose fine extent is not twice the coarse one (odd
 * ghost depth), mixed sizes, or an out-of-range index. */
int mhdvlct_refresh_faces(mhdvlct_handle* h, const MhdBlockView* blocks, int nblocks,
                          const MhdRefreshFace* faces, int nfaces,
                          unsigned conservative, void* stream);

/* Flux correction at coarse-fine faces: Cello's "flux_correct" Method, run
 * after a step whose boundary fluxes were stored (mhdvlct_block_step_fc):
 *   - each finer block's stored fluxes through its face toward a coarser
 *     neighbour are coarsened onto that neighbour's face
 *     (FaceFluxes::coarsen, src/Cello/data_FaceFluxes.cpp:128-252) and
 *     summed (FluxData::sum_neighbor_fluxes, data_FluxData.hpp:132-145);
 *   - the coarse block's boundary cells on such faces get
 *     (2 face - 1) (own flux - neighbour flux) added, density first, the
 *     `conservative` fields as density-weighted values divided by the
 *     corrected density (MethodFluxCorrect::flux_correct_,
 *     src/Cello/problem_MethodFluxCorrect.cpp:293-558).
 * fluxes: one MhdFluxCorrection per block (host array of device pointers)
 * holding the fluxes the step stored; every block stores the same
 * quantities.  faces: the mesh's refresh faces (mhdvlct_refresh_faces); the
 * axis faces of type MHD_REFRESH_COARSE are the ones used.  Cell fields
 * updated: density, velocity_x/y/z (momentum fluxes), total_energy,
 * internal_energy and the passive scalars, as stored; a passive scalar in
 * the `conservative` mask (bit MHD_FIELD_PASSIVE_0 + k) is corrected as a
 * density-weighted value like the velocities. */
int mhdvlct_flux_correct(mhdvlct_handle* h, const MhdBlockView* blocks, int nblocks,
                         const MhdFluxCorrection* fluxes, const MhdRefreshFace* faces,
                         int nfaces, unsigned conservative, void* stream);

/* The regions of one face (host only, no device work): the sender's cells
 * read (send_start/send_size, array indices of the sender) and the
 * receiver's ghost cells written (recv_start/recv_size), as Cello's Box
 * computes them (src/Cello/mesh_Box.cpp:13-234) for a field of the given
 * centering.  Returns 1 when the face has cells to refresh, 0 when not, and
 * a negative value on a bad argument. */
int mhdvlct_refresh_face_box(const int n[3], const int ghost[3], const int centering[3],
                             int type, const int face[3], const int child[3],
                             int send_start[3], int send_size[3], int recv_start[3],
                             int recv_size[3]);

/* ------------------------------------------------------------- batch
 * Many blocks of possibly different sizes advanced together: one fused,
 * persistent launch per stage over all blocks, the cycle captured as a CUDA
 * graph.  Library-owned state; the caller reads/writes it through
 * mhdvlct_batch_block_view (device pointers). */
typedef struct mhdvlct_batch mhdvlct_batch;

/* dims: nblocks x 3 active extents; widths: nblocks x 3 cell widths;
 * ghost: ghost depth of every block; dtype: MHD_DTYPE_*. */
int mhdvlct_batch_create(mhdvlct_handle* h, const int* dims,
                         const double* widths, int nblocks, int ghost,
                         int dtype, mhdvlct_batch** out);
/* As mhdvlct_batch_create, with npassive (0..4) passive scalars in
 * conserved form and, with gravity = 1, acceleration_x/y/z fields in every
 * block (MhdBlockView::passive / acceleration of mhdvlct_batch_block_view):
 * the scalars are advected and the gravity source is added on the full-dt
 * stage exactly as mhdvlct_block_step does, and the refresh covers both, as
 * Cello refreshes every field (EnzoMethodMHDVlct.cpp:146-151).  The
 * acceleration is the caller's: no step writes it. */
int mhdvlct_batch_create_ex(mhdvlct_handle* h, const int* dims,
                            const double* widths, int nblocks, int ghost,
                            int dtype, int npassive, int gravity,
                            mhdvlct_batch** out);
int mhdvlct_batch_destroy(mhdvlct_batch* b);
/* Device pointers of block i's current state (valid until the next step). */
int mhdvlct_batch_block_view(mhdvlct_batch* b, int i, MhdBlockView* out);
/* nbr: nblocks x 27 block indices, nbr[27*i + (sz+1)*9 + (sy+1)*3 + (sx+1)]
 * supplies the ghost region at offset (sx, sy, sz) of block i (same-size
 * neighbours).  Default: every block is periodic on itself. */
int mhdvlct_batch_set_neighbors(mhdvlct_batch* b, const int* nbr);
/* Ghost refresh of every block from its neighbours. */
int mhdvlct_batch_refresh(mhdvlct_batch* b, void* stream);
/* Replace the batch's same-level refresh by the mesh refresh of `faces`
 * (block indices of the batch; see mhdvlct_refresh_faces), planned once and
 * replayed inside the cycle's CUDA graph.  nfaces = 0 restores the
 * 27-neighbour refresh.  Every block must have the same extents. */
int mhdvlct_batch_set_refresh_faces(mhdvlct_batch* b, const MhdRefreshFace* faces,
                                    int nfaces, unsigned conservative);
/* Store the boundary fluxes of `quantities` (bits of MHD_Q_*) on the final
 * stage of every cycle and apply the flux correction of the mesh `faces`
 * (see mhdvlct_flux_correct) right after it, inside the cycle's CUDA graph:
 * the reference's Method list ["mhd_vlct", "flux_correct"].  Hydro only;
 * blocks of equal extents; bit MHD_Q_PASSIVE_0 + k needs the batch's
 * npassive > k.  quantities = 0 turns it off. */
int mhdvlct_batch_set_flux_correction(mhdvlct_batch* b, unsigned quantities,
                                      const MhdRefreshFace* faces, int nfaces,
                                      unsigned conservative);
/* One VL+CT step of every block; dt_per_block: host array of nblocks. */
int mhdvlct_batch_step(mhdvlct_batch* b, const double* dt_per_block,
                       void* stream);
/* Per-block courant-limited dt (reference semantics, whole ghosted block);
 * dt_out: host array of nblocks.  Synchronises the stream. */
int mhdvlct_batch_timestep(mhdvlct_batch* b, double* dt_out, void* stream);
/* Advance ncycles full cycles (timestep, refresh, two stages) entirely on
 * the device: dt_mode 0 = one global dt (Cello's min-reduction), 1 = each
 * block its own dt.  The cycle is captured once as a CUDA graph and
 * replayed.  elapsed_time_out (may be NULL) receives the sum of dt. */
int mhdvlct_batch_run(mhdvlct_batch* b, int ncycles, int dt_mode,
                      double* elapsed_time_out, void* stream);
/* Work decomposition: tile extent used per block size class (0 = auto). */
int mhdvlct_batch_set_tile(mhdvlct_batch* b, int tile_x, int tile_y);
/* One stage's work decomposition for every block (stage 0: half dt, 1: full
 * dt): tile extents, z-chunk length (0 = whole block) and CTA size (256, or
 * 512 where the stage allows it; 0 = 256), e.g. to pin a tuned choice. */
int mhdvlct_batch_set_stage_tile(mhdvlct_batch* b, int stage, int tile_x,
                                 int tile_y, int zchunk, int threads);
/* The autotuner: for every block-size class, time candidate (tile, z-chunk)
 * work decompositions on the batch's own data and keep the fastest.  The
 * state is restored afterwards.  json_out (may be NULL) receives a JSON
 * description of the choices. */
int mhdvlct_batch_autotune(mhdvlct_batch* b, int reps, char* json_out,
                           size_t json_len, void* stream);
/* Device address and size of the contiguous region holding every block's
 * state (cell fields and both face-B buffers), for bulk host transfers. */
int mhdvlct_batch_state_region(mhdvlct_batch* b, void** dev_ptr,
                               size_t* bytes);
/* Conserved totals and constraint diagnostics of the current state over the
 * active zones of every block, accumulated on the device in FP64 (whatever
 * the storage precision) in a fixed order, so bit-reproducible:
 * out[0] mass, out[1..3] momentum, out[4] total energy (sum rho e_tot dV),
 * out[5] sum rho e_int dV (dual energy, else 0), out[6] max |div B| over
 * cells (from the face-centred B), out[7] max |B| at cell centres.
 * Synchronises the stream.  (The reference computes such sums in its
 * analysis scripts; no Method counterpart.) */
int mhdvlct_batch_diagnostics(mhdvlct_batch* b, double* out, void* stream);
/* The current state only (every block's cell fields and its current face-B
 * buffer), as one or two contiguous device segments: dev_ptrs[i] / bytes[i]
 * for i < *nsegments (max_segments >= 2).  Valid until the next step; what a
 * host that keeps the fields transfers each cycle. */
/* Advance ncycles with the state held in pinned host memory: `host` holds
 * every block's cell fields, then every block's current face B, back to back
 * (the segments of mhdvlct_batch_state_segments, `bytes` their total).  Every
 * cycle copies the state in, runs the cycle with one global dt and copies
 * the new state back out -- Cello's host-resident field data.  The copies
 * are pipelined with the full-dt stage by `ngroups` groups of consecutive
 * blocks: a group's new state leaves as soon as its stage is done and, when
 * another cycle follows, comes straight back in while later groups still
 * compute.  The stream completes when the final state is in `host`;
 * elapsed_out (may be NULL) receives the simulated time advanced. */
int mhdvlct_batch_run_host(mhdvlct_batch* b, void* host, size_t bytes, int ncycles,
                           int ngroups, double* elapsed_out, void* stream);
int mhdvlct_batch_state_segments(mhdvlct_batch* b, void** dev_ptrs, size_t* bytes,
                                 int max_segments, int* nsegments);
/* Run `reps` cycles as individual launches with CUDA events between the
 * kernels; ms_out[0..4] = mean ms per cycle of the timestep reduction, the
 * ghost refresh, stage 1 (half dt), stage 2 (full dt) and the whole cycle. */
int mhdvlct_batch_profile(mhdvlct_batch* b, int reps, int dt_mode,
                          float* ms_out, void* stream);

/* ------------------------------------------------------------- serving
 * Continuous batching of independent solves (each a periodic box of n^3
 * cells), admitted against a device-memory budget. */
typedef struct mhdserve mhdserve;
typedef struct MhdServeRequest {
  int n;                      /* active cells per side                      */
  int cycles;                 /* number of VL+CT cycles                     */
  char riemann_solver[16];
  char reconstruct_method[16];
  int mhd;                    /* 1: constrained_transport, 0: no_bfield     */
  double box_size;            /* physical side length                       */
  /* Initial state as float32 host arrays in the ghosted block layout of an
   * n^3 block with 3 ghost layers (copied by mhdserve_submit): density,
   * velocity_x/y/z, total_energy and, with mhd, bfield_x/y/z and
   * bfieldi_x/y/z.  The ghost zones are refreshed periodically on admission. */
  const float* init[12];
} MhdServeRequest;

int mhdserve_create(const MhdVlctParams* base, size_t hbm_budget_bytes,
                    int max_active, mhdserve** out);
int mhdserve_destroy(mhdserve* s);
/* Queue a request; returns its ticket.  Rejected (MHD_ERR_NOMEM) if it could
 * never fit in the budget, MHD_ERR_INVALID if malformed. */
int mhdserve_submit(mhdserve* s, const MhdServeRequest* r, int* ticket);
/* Run the scheduler for up to max_iterations iterations (one cycle of every
 * active request per iteration); admits queued requests as memory frees. */
int mhdserve_pump(mhdserve* s, int max_iterations);
/* 0 = queued, 1 = running, 2 = done, 3 = failed */
int mhdserve_poll(mhdserve* s, int ticket, int* state);
/* Copy the final state (density, vx, vy, vz, etot[, bx, by, bz]) of a done
 * request into host arrays of n^3 active cells each. */
int mhdserve_result(mhdserve* s, int ticket, float* const* out_fields,
                    double* sim_time_out);
/* Host wall-clock seconds (steady clock) of a request's submission,
 * admission and completion. */
int mhdserve_timing(mhdserve* s, int ticket, double* t_submit, double* t_admit,
                    double* t_done);
const char* mhdserve_last_error_string(const mhdserve* s);

#ifdef __cplusplus
}
#endif
#endif /* MHDVLCT_GB300_H */
