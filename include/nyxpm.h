/*
 * nyxpm.h -- C ABI of the GB300-native particle-mesh (PM) gravity step for Nyx.
 *
 * One periodic, single-level, dark-matter-only grid ("box") per handle.  All
 * particle and field state stays resident in GPU memory between calls; host
 * buffers cross the boundary only in the upload / download calls and in the
 * optional output pointers.  Every call is enqueued on the context's CUDA stream;
 * calls that return host data synchronise that stream.  No call aborts the
 * process: each returns an nyxpm_status and nyxpm_last_error() gives the text.
 * One host thread per context.
 *
 * Each entry point names the Nyx interface it replaces (paths inside the Nyx
 * source tree).  The plain FP64 form computes exactly what those routines
 * compute on a periodic single level; the restated pieces that live in AMReX
 * (CIC deposit, MLMG) follow the definitions written next to each call.
 */
#ifndef NYXPM_H
#define NYXPM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NYXPM_ABI_VERSION 2

typedef enum nyxpm_status {
    NYXPM_OK = 0,
    NYXPM_INVALID_ARG = 1,    /* bad size, null pointer, unsupported grid */
    NYXPM_OOM = 2,            /* device memory exhausted */
    NYXPM_CUDA_ERROR = 3,     /* a CUDA runtime call or kernel failed */
    NYXPM_NOT_CONVERGED = 4,  /* multigrid hit max_vcycles above tolerance */
    NYXPM_TIMEOUT = 5,        /* a bounded device wait ran out */
    NYXPM_NO_DEVICE = 6       /* no usable CUDA device */
} nyxpm_status;

/* Precision of a box's particle and field storage. */
typedef enum nyxpm_precision {
    NYXPM_FP64 = 0,           /* plain drop-in: FP64 everywhere */
    NYXPM_MIXED = 1           /* FP32 cell-relative positions, FP32 deposit and V-cycles
                                 inside FP64 defect correction */
} nyxpm_precision;

/* Flags of nyxpm_step. */
#define NYXPM_STEP_REUSE_FIELD 1u  /* take the old-time field from the previous step's
                                      new-time solve (one deposit + one solve per step)
                                      instead of re-solving from the start-of-step
                                      positions with a zero guess */

typedef struct nyxpm_params {
    int device;             /* CUDA device ordinal */
    void* stream;           /* cudaStream_t to enqueue on; NULL: the context creates one */
    double comoving_OmM;    /* nyx.comoving_OmM */
    double comoving_OmR;    /* nyx.comoving_OmR */
    double comoving_h;      /* nyx.comoving_h */
    double gconst;          /* Gconst in code units (Mpc, M_sun, km/s) */
    double rel_tol;         /* gravity.sl_tol / gravity.ml_tol */
    int max_vcycles;        /* V-cycle limit per solve */
    int nu1, nu2;           /* red-black Gauss-Seidel sweeps before / after the coarse correction */
    int verbose;
    int mixed_inner_vcycles;/* NYXPM_MIXED: FP32 V-cycles per FP64 defect-correction iteration */
    int mg_fused_edge;      /* the FP32 V-cycle levels of at most this many cells per edge
                               (the FP64 ones of at most half as many, below the finest) run
                               as one launch (one CTA per box) per V-cycle, same results;
                               0: one launch per pass on every level (default 16) */
} nyxpm_params;

typedef struct nyxpm_ctx nyxpm_ctx;
typedef struct nyxpm_box nyxpm_box;

/* Result of one solve (Gravity::solve_for_phi stores the final residual norm in
 * level_solver_resnorm, Source/Gravity/Gravity.cpp:312-314). */
typedef struct nyxpm_solve_info {
    int vcycles;            /* V-cycles (FP64) or outer defect-correction iterations (mixed) */
    int inner_vcycles;      /* FP32 V-cycles inside the defect correction (mixed only) */
    double resnorm0;        /* ||rhs - L phi0||_inf */
    double resnorm;         /* ||rhs - L phi||_inf at exit */
    double bnorm;           /* ||rhs||_inf */
} nyxpm_solve_info;

typedef struct nyxpm_step_info {
    nyxpm_solve_info old_solve;   /* zeroed when the old-time field was reused */
    nyxpm_solve_info new_solve;
} nyxpm_step_info;

/* ---- context ---------------------------------------------------------------- */

/* Defaults: device 0, own stream, Einstein-de Sitter with h = 0.675, Gconst of
 * Source/Driver/constants_cosmo.H:15-16, rel_tol 1e-10, 100 V-cycles, nu1 = nu2 = 2. */
void nyxpm_default_params(nyxpm_params* p);

/* Replaces Gravity::Gravity (Source/Gravity/Gravity.cpp:49-68) and the particle
 * container construction of Nyx::init_particles (Source/Particle/NyxParticles.cpp:378). */
nyxpm_status nyxpm_create(const nyxpm_params* p, nyxpm_ctx** out);
void nyxpm_destroy(nyxpm_ctx* ctx);
const char* nyxpm_last_error(const nyxpm_ctx* ctx);
int nyxpm_abi_version(void);
/* The CUDA stream the context enqueues on (cudaStream_t). */
void* nyxpm_stream(nyxpm_ctx* ctx);
nyxpm_status nyxpm_synchronize(nyxpm_ctx* ctx);

/* ---- boxes ------------------------------------------------------------------ */

/* A periodic n^3 grid of side L (prob_lo = 0) holding up to np particles.
 * n must be m * 2^k with m <= 8 (the multigrid coarsens by 2 down to m^3).
 * All device memory the box needs is allocated here; no later call allocates. */
nyxpm_status nyxpm_box_create(nyxpm_ctx* ctx, int n, double L, int64_t np,
                              nyxpm_precision prec, nyxpm_box** out);
nyxpm_status nyxpm_box_destroy(nyxpm_ctx* ctx, nyxpm_box* box);
/* Device bytes held by a box of this shape (for admission by memory budget). */
size_t nyxpm_box_bytes(int n, int64_t np, nyxpm_precision prec);

/* Particle state in: pos and vel are np x 3 (x, y, z per particle), mass is np
 * values or NULL for a uniform mass_scalar.  Particle ids are the row indices.
 * (Replaces the AsciiFile/BinaryFile/cosmological fills of init_particles,
 * Source/Particle/NyxParticles.cpp:378-591.) */
nyxpm_status nyxpm_box_upload(nyxpm_ctx* ctx, nyxpm_box* box, const double* pos,
                              const double* vel, const double* mass, double mass_scalar);
/* Particle state out, in id order (row i = the particle uploaded in row i). */
nyxpm_status nyxpm_box_download(nyxpm_ctx* ctx, nyxpm_box* box, double* pos, double* vel);

/* Gravity::set_mass_offset (Source/Gravity/Gravity.cpp:975-1030) with
 * NyxParticleContainer::sumParticleMass (Source/Particle/NyxParticleContainer.H:70-79):
 * mass_offset = sum(m) / L^3.  Called by nyxpm_box_upload; returns the value. */
nyxpm_status nyxpm_set_mass_offset(nyxpm_ctx* ctx, nyxpm_box* box, double* mass_offset);

/* ---- the hot path -------------------------------------------------------------- */

/* Periodic shift of positions into [0, L) and counting sort by deposit cell.
 * Replaces NyxParticleContainer::RedistributeLocal (Source/Particle/NyxParticleContainer.H:123-136,
 * called from Nyx::post_timestep, Source/Driver/Nyx.cpp:1421-1437).  Deterministic:
 * equal keys keep their previous relative order. */
nyxpm_status nyxpm_redistribute(nyxpm_ctx* ctx, nyxpm_box* box);

/* CIC mass density of the particles (sorted first).  Replaces
 * NyxParticleContainer::AssignDensitySingleLevel / AssignDensity
 * (Source/Particle/NyxParticleContainer.H:90-97 -> AMReX AssignCellDensitySingleLevel;
 * restated in-tree at Source/Particle/NeutrinoParticleContainer.cpp:160-320).
 * The density stays on the device for nyxpm_solve_phi; rho_out (n^3, x fastest)
 * may be NULL. */
nyxpm_status nyxpm_deposit(nyxpm_ctx* ctx, nyxpm_box* box, double* rho_out);

/* Gravity::solve_for_phi (Source/Gravity/Gravity.cpp:267-315): RHS = -4 pi G
 * (rho - mass_offset - mean) / a from the last deposit, then multigrid V-cycles
 * to ||r||_inf <= rel_tol * max(||rhs||_inf, ||r0||_inf).  zero_guess = 1 starts
 * from phi = 0 (actual_multilevel_solve with use_previous_phi_as_guess = 0,
 * Gravity.cpp:665-666); 0 starts from the current phi.  info may be NULL. */
nyxpm_status nyxpm_solve_phi(nyxpm_ctx* ctx, nyxpm_box* box, double a, int zero_guess,
                             nyxpm_solve_info* info);

/* phi (PhiGrav_Type, n^3 x fastest) out / in. */
nyxpm_status nyxpm_get_phi(nyxpm_ctx* ctx, nyxpm_box* box, double* phi);
nyxpm_status nyxpm_set_phi(nyxpm_ctx* ctx, nyxpm_box* box, const double* phi);

/* Cell-centred gravity vector g = average of the two face gradients of phi
 * (Gravity::get_new_grav_vector, Source/Gravity/Gravity.cpp:817-850).  g_out
 * receives 3 n^3 values, component-major; it may be NULL (the field then stays
 * on the device). */
nyxpm_status nyxpm_grav_vector(nyxpm_ctx* ctx, nyxpm_box* box, double* g_out);

/* The caller's acceleration for the next kicks: the `acc` MultiFab argument of
 * DarkMatterParticleContainer::moveKickDrift / moveKick
 * (Source/Particle/DarkMatterParticleContainer.cpp:76-112, 184-247;
 * NyxParticleContainer.H:15-18), e.g. the grav_vec_old / grav_vec_new that Nyx's
 * own Gravity object computed.  g holds 3 n^3 values, component-major, x fastest:
 * the valid cells of a cell-centred 3-component field on the box's grid (the
 * kicks wrap the CIC corners periodically, which is what the reference's
 * periodic ghost fill of acc gives).  on_device = 0: g is host memory, copied
 * before the call returns; 1: g is device memory on the context's device, copied
 * on the context's stream.  The field replaces the box's own gravity vector until
 * the next solve (nyxpm_solve_phi, nyxpm_step, nyxpm_init_field, nyxpm_set_phi);
 * mixed boxes round it to FP32 as their kicks read it. */
nyxpm_status nyxpm_set_grav_vector(nyxpm_ctx* ctx, nyxpm_box* box, const double* g, int on_device);

/* DarkMatterParticleContainer::moveKickDrift (Source/Particle/DarkMatterParticleContainer.cpp:76-181):
 * the box's cell-centred gravity vector (kept in step with phi, or the caller's
 * from nyxpm_set_grav_vector) interpolated to the particle by CIC,
 * v = (a_old v + dt/2 g)/a_half, x += dt/a_half v
 * (update_dm_particle_single, :250-306, do_move = 1). */
nyxpm_status nyxpm_kick_drift(nyxpm_ctx* ctx, nyxpm_box* box, double dt, double a_old,
                              double a_half);

/* DarkMatterParticleContainer::moveKick (:184-247): v = (a_half v + dt/2 g)/a_new. */
nyxpm_status nyxpm_kick(nyxpm_ctx* ctx, nyxpm_box* box, double dt, double a_new, double a_half);

/* One PM step of Nyx::advance_particles_only on level 0
 * (Source/TimeStep/Nyx_advance_particles.cpp:137-268) plus the periodic shift of
 * Nyx::post_timestep: [old-time deposit + solve], kick-drift, deposit, new-time
 * solve (old phi as guess), kick, wrap.  a_half = (a_old + a_new)/2.  flags:
 * NYXPM_STEP_REUSE_FIELD.  info may be NULL. */
nyxpm_status nyxpm_step(nyxpm_ctx* ctx, nyxpm_box* box, double a_old, double a_new, double dt,
                        unsigned flags, nyxpm_step_info* info);

/* nyxpm_box_upload + nyxpm_step + nyxpm_box_download in one call, for callers
 * whose particles live in host memory; pos and vel (np x 3, particle order) are
 * read and overwritten with the stepped state.  The results are those of the
 * three calls, bit for bit.  The transfers run on a second stream under the
 * step (both precisions): the velocities arrive during the sort, deposit and
 * old-time solve, which read positions only, and the positions leave (wrapped,
 * as the closing kick wraps them) during the new-time deposit and solve.
 * Pinned host buffers let the copies overlap.  No counterpart in the
 * reference: Nyx keeps the particles in its own containers. */
nyxpm_status nyxpm_step_host(nyxpm_ctx* ctx, nyxpm_box* box, double* pos, double* vel,
                             const double* mass, double mass_scalar, double a_old, double a_new,
                             double dt, unsigned flags, nyxpm_step_info* info);

/* The post_init solve (Nyx::post_init, Source/Driver/Nyx.cpp:1957-2005):
 * redistribute, deposit, solve from phi = 0 at scale factor a. */
nyxpm_status nyxpm_init_field(nyxpm_ctx* ctx, nyxpm_box* box, double a, nyxpm_solve_info* info);

/* ---- a(t), FP64 on the host (Source/Driver/comoving.cpp) -------------------------- */

/* Nyx::integrate_comoving_a(old_a, new_a, dt), comoving.cpp:629-688. */
double nyxpm_integrate_a(const nyxpm_params* p, double a_old, double dt);
/* Nyx::integrate_comoving_a_to_a, comoving.cpp:74-130 (dt_window = search window). */
double nyxpm_dt_for_da(const nyxpm_params* p, double a_old, double a_value, double dt_window);

/* ---- time-step control ---------------------------------------------------------- */

/* The inputs of Nyx's level-0 time-step choice (names of the reference's
 * parameters; defaults from nyxpm_default_dt_params are the reference's). */
typedef struct {
    double cfl;                   /* particles.cfl (NyxParticles.cpp:152), 0.5 */
    double change_max;            /* nyx.change_max (Nyx.cpp:83), 1.1; dt <= change_max * dt_old */
    double relative_max_change_a; /* nyx.relative_max_change_a (comoving.cpp:10), 0.01 */
    double absolute_max_change_a; /* nyx.absolute_max_change_a (comoving.cpp:11), -1 = off */
    double final_a;               /* nyx.final_a (comoving.cpp:8), -1 = off */
    double stop_time;             /* stop_time, -1 = off */
    double dt_binpow;             /* nyx.dt_binpow (comoving.cpp:12), -1 = off */
} nyxpm_dt_params;

void nyxpm_default_dt_params(nyxpm_dt_params* dp);

/* Particle time-step limit, replaces NyxParticleContainer::estTimestep
 * (Source/Particle/NyxParticleContainer.H:329-465) as called from
 * Nyx::particle_est_time_step (NyxParticles.cpp:1027-1067): the minimum over
 * particles of cfl / max_d(|v_d| / (a dx)) and 1 / sqrt(|g| / dx), g the
 * box's current gravity vector at the particle's cell.  *dt = 1e50 when no
 * particle limits it, -1e50 when the box has no particles.  One GPU reduction;
 * the box must hold a field (after a solve, a step or nyxpm_set_phi). */
nyxpm_status nyxpm_est_time_step(nyxpm_ctx* ctx, nyxpm_box* box, double cfl, double a, double* dt);

/* Nyx::comoving_est_time_step (Source/Driver/comoving.cpp:353-483) from scale
 * factor a: limits estdt by how fast a may change (estdt_comoving_a and its
 * helpers, :191-350).  Host FP64.  NYXPM_INVALID_ARG where the reference
 * aborts (a > final_a, no convergence in 100 iterations). */
nyxpm_status nyxpm_comoving_est_dt(const nyxpm_params* p, double a, double estdt,
                                   const nyxpm_dt_params* dp, double* dt);

/* Nyx::computeNewDt at level 0 without subcycling (Source/Driver/Nyx.cpp:1023-1208):
 * est_time_step (particles, then the a-change limit; Nyx.cpp:912-1020), then
 * dt <= change_max * dt_old (skipped when dt_old <= 0, the first step), then
 * the stop_time clip; *a_new = a advanced by the chosen dt. */
nyxpm_status nyxpm_compute_new_dt(nyxpm_ctx* ctx, nyxpm_box* box, const nyxpm_dt_params* dp,
                                  double time, double a, double dt_old, double* dt_new,
                                  double* a_new);

/* ---- particle files and the comoving_a file (host I/O) ---------------------------- */

/* Nyx's particle initial-condition files (nyx.particle_init_type, read by
 * Nyx::init_particles, Source/Particle/NyxParticles.cpp:506-560; formats of
 * Docs/sphinx_documentation/source/ICs.rst:13-78):
 *   ASCII        first line the particle count, then "x y z mass vx vy vz" per line;
 *   BINARY       int64 NP, int32 DM = 3, int32 NX >= 4, then NP records of DM + NX
 *                float32 or float64 values "x y z mass vx vy vz [extras]" (the
 *                precision follows from the file size);
 *   BINARY_META  a text file listing BINARY files, one per line, read in order. */
typedef enum {
    NYXPM_FILE_ASCII = 0,
    NYXPM_FILE_BINARY = 1,
    NYXPM_FILE_BINARY_META = 2,
    NYXPM_FILE_BINARY_F64 = 3     /* BINARY written with float64 records (read as BINARY) */
} nyxpm_file_format;

/* Number of particles the file holds (reads only the headers). */
nyxpm_status nyxpm_particle_file_count(const char* path, nyxpm_file_format fmt, int64_t* np,
                                       char* errbuf, size_t errlen);
/* Reads the particles into host arrays laid out as nyxpm_box_upload takes them:
 * pos[3 np], vel[3 np], mass[np].  capacity = the arrays' particle count. */
nyxpm_status nyxpm_particle_file_read(const char* path, nyxpm_file_format fmt, int64_t capacity,
                                      double* pos, double* vel, double* mass, int64_t* np_read,
                                      char* errbuf, size_t errlen);
/* Writes an ASCII (17 significant digits), BINARY (float32) or BINARY_F64
 * (float64, exact) particle file; mass NULL writes mass_scalar for every particle. */
nyxpm_status nyxpm_particle_file_write(const char* path, nyxpm_file_format fmt, int64_t np,
                                       const double* pos, const double* vel, const double* mass,
                                       double mass_scalar, char* errbuf, size_t errlen);
/* The comoving_a file of a checkpoint or plotfile directory: written as
 * Nyx::checkPointPost does (Source/IO/Nyx_output.cpp:994-1010, 15 significant
 * digits), read as Nyx::comoving_a_post_restart does (comoving.cpp:690-705). */
nyxpm_status nyxpm_write_comoving_a(const char* dir, double a, char* errbuf, size_t errlen);
nyxpm_status nyxpm_read_comoving_a(const char* dir, double* a, char* errbuf, size_t errlen);

/* Nyx's one-particle-per-cell cosmological ICs on a single level
 * (DarkMatterParticleContainer::InitCosmo1ppcMultiLevel,
 * Source/Particle/DarkMatterParticleContainer.cpp:309-450, called by Nyx::initcosmo,
 * Source/Initialization/Nyx_initcosmo.cpp:100-427).  The particle of cell (i, j, k)
 * sits at ((i + 1/2) dx + disp_x(i,j,k) * disp_fac[0], ...), shifted periodically
 * into [0, L), with velocity vel_d(i,j,k) * vel_fac[d].  disp and vel hold 3 n^3
 * values each, one component after another, x fastest: the displacement and
 * velocity components of the IC MultiFab.  pos_out / vel_out: n^3 x 3.  Host only. */
nyxpm_status nyxpm_cosmo_1ppc_particles(int n, double L, const double* disp, const double* vel,
                                        const double* disp_fac, const double* vel_fac,
                                        double* pos_out, double* vel_out);
/* The factors and the particle mass Nyx::initcosmo takes for an IC source
 * (Nyx_initcosmo.cpp:185-294), dark matter only: source 0 = MUSIC (disp_fac = L,
 * vel_fac = L h, mass = rho_m dx^3), 1 = nyx (disp_fac = L,
 * vel_fac = L a sqrt(OmM / a^3 + 1 - OmM) 100 h with a = 1 / (1 + redshift),
 * mass = rho_m L^3 / n^3); rho_m = 3 (100 h)^2 OmM / (8 pi G). */
nyxpm_status nyxpm_cosmo_ic_factors(const nyxpm_params* p, int source, int n, double L,
                                    double redshift, double* disp_fac, double* vel_fac,
                                    double* particle_mass);
/* nyxpm_cosmo_1ppc_particles into the box (np must be n^3) with the uniform
 * particle mass, as nyxpm_box_upload. */
nyxpm_status nyxpm_box_init_cosmo_1ppc(nyxpm_ctx* ctx, nyxpm_box* box, const double* disp,
                                       const double* vel, const double* disp_fac,
                                       const double* vel_fac, double particle_mass);

/* ---- checkpoint and plotfile particle directories (host I/O) ---------------------- */

/* The "DM" directory of a Nyx checkpoint (chkNNNNN/DM, written by NyxCheckpoint,
 * Source/Particle/NyxParticleContainer.H:510-517, from Nyx::particle_check_point,
 * Source/IO/Nyx_output.cpp:726-750) or plotfile (pltNNNNN/DM, WriteNyxPlotFile,
 * NyxParticleContainer.H:499-505): the AMReX particle container layout
 * Version_Two_Dot_Zero -- a text Header (version and real precision, dimension,
 * the names of the real and int components, checkpoint flag, particle count,
 * next id, finest level, grids per level, one "file count offset" line per
 * grid), binary Level_<l>/DATA_<nnnnn> files (per grid: a checkpoint's int32 id
 * and cpu, then x y z and the real components per particle, native byte order)
 * and Level_<l>/Particle_H (the level's BoxArray).  Nyx reads it back with
 * Restart (Source/Particle/NyxParticles.cpp:584-586, 928-934). */
typedef struct nyxpm_particle_header {
    int single_precision;   /* Version_Two_Dot_Zero_single: float32 reals; 0: float64 */
    int dim;                /* 3 */
    int n_real_extra;       /* real components after the position (Nyx DM: 4) */
    int n_int_extra;        /* int components after id and cpu */
    int is_checkpoint;      /* 1: ids and cpus stored (checkpoint); 0: plotfile */
    int finest_level;
    int64_t num_particles;
    int64_t max_next_id;
    int ngrids;             /* grids over all levels */
    int pad;
} nyxpm_particle_header;

nyxpm_status nyxpm_particles_info(const char* dir, nyxpm_particle_header* h, char* errbuf,
                                  size_t errlen);
/* Every grid of every level in header order into pos[3 np], vel[3 np], mass[np]
 * (the arrays nyxpm_box_upload takes); mass and velocity are the components named
 * mass, xvel, yvel, zvel (else the first four); ids (may be NULL; checkpoints
 * only) receives the AMReX particle ids. */
nyxpm_status nyxpm_particles_read(const char* dir, int64_t capacity, double* pos, double* vel,
                                  double* mass, int64_t* ids, int64_t* np_read, char* errbuf,
                                  size_t errlen);
/* Writes dir (created if absent) as one level with one grid covering the n^3
 * periodic domain: ids 1..np, cpu 0, components mass xvel yvel zvel; float32
 * reals with single_precision, float64 otherwise; mass NULL writes mass_scalar. */
nyxpm_status nyxpm_particles_write(const char* dir, int n, int64_t np, const double* pos,
                                   const double* vel, const double* mass, double mass_scalar,
                                   int is_checkpoint, int single_precision, char* errbuf,
                                   size_t errlen);

/* ---- AMReX MultiFab files (VisMF, host I/O) ------------------------------------ */

/* A cell-centred MultiFab stored as VisMF::Write stores it, header version 1:
 * <name>_H (version, write mode, ncomp, ngrow, the BoxArray, one
 * "FabOnDisk: <file> <offset>" per box, per-box per-component min and max) and
 * data files holding each FAB as a text header (real descriptor, box, ncomp)
 * and its values, component after component, x fastest.  This is the form of
 * the IC MultiFab <cosmo.initDirName>/Level_0/Cell that Nyx::icReadAndPrepareFab
 * reads with VisMF::Read (Source/Initialization/Nyx_initcosmo.cpp:15-96). */
typedef struct nyxpm_multifab_info {
    int ncomp;
    int ngrow;
    int nboxes;
    int lo[3], hi[3];      /* bounding box of the BoxArray (cell indices) */
    int has_minmax;        /* the header holds the min/max tables */
} nyxpm_multifab_info;

#define NYXPM_MF_REJECT_NAN 1u   /* a NaN is an error, as icReadAndPrepareFab's check */

nyxpm_status nyxpm_multifab_info_read(const char* name, nyxpm_multifab_info* info, char* errbuf,
                                      size_t errlen);
/* boxes_out: nboxes x 6 ints (lo x y z, hi x y z) in header order; minmax_out:
 * nboxes x ncomp x (min, max) from the header.  Either may be NULL. */
nyxpm_status nyxpm_multifab_boxes(const char* name, int* boxes_out, double* minmax_out,
                                  char* errbuf, size_t errlen);
/* Components [comp0, comp0 + ncomp) of the valid cells in [lo, hi] into out
 * (ncomp blocks of nx ny nz values, x fastest).  Every cell of [lo, hi] must lie
 * in exactly one box.  FABs of IEEE float64 or float32 in either byte order. */
nyxpm_status nyxpm_multifab_read(const char* name, int comp0, int ncomp, const int* lo,
                                 const int* hi, unsigned flags, double* out, char* errbuf,
                                 size_t errlen);
/* Writes data (ncomp blocks over [lo, hi], x fastest) as a MultiFab with ngrow 0:
 * the boxes given (nboxes x 6 ints that tile [lo, hi]) or, with boxes NULL, the
 * region cut into boxes of at most max_grid_size cells per edge (x fastest,
 * then y, then z).  One data file <name>_D_00000, float64 in the host's byte
 * order.  The directory of name must exist. */
nyxpm_status nyxpm_multifab_write(const char* name, int ncomp, const int* lo, const int* hi,
                                  int max_grid_size, int nboxes, const int* boxes,
                                  const double* data, char* errbuf, size_t errlen);

/* ---- ensembles and serving ------------------------------------------------------ */

/* An ensemble holds many independent periodic boxes of uneven sizes in the
 * mixed-precision form and advances them together: every stage of a step is one
 * persistent launch over a work list spanning all boxes, and the step is
 * replayed from captured CUDA graphs.  Box memory comes from a device arena of
 * a fixed byte budget allocated at creation, so boxes can be added and removed
 * between steps (continuous batching) without further device allocation.  No
 * counterpart in the reference: Nyx runs one simulation per process. */
typedef struct nyxpm_ensemble nyxpm_ensemble;

/* Shapes chosen by the autotuner (nyx_gb300/autotune.py). */
typedef struct nyxpm_tuning {
    int deposit_tile;       /* 0: 8x8x8 cells, 1: 8x8x4, 2: 16x8x4 */
    int smooth_rows;        /* plane rows per multigrid work item: 1, 2, 4 or 8 */
    int inner_vcycles;      /* FP32 V-cycles per FP64 defect-correction iteration */
    int max_outer;          /* defect-correction iterations inside the step graph */
    int sort_bucket;        /* particles per work item of the sort and the kicks: 256, 512 or 1024 */
    int prolong_quad;       /* 1: the black-only prolongation covers four fine rows (2 x 2) per
                               task, sharing the coarse rows; 0: one fine row per task */
} nyxpm_tuning;

typedef struct nyxpm_ensemble_info {
    int boxes;              /* boxes stepped */
    int max_outer_used;     /* most defect-correction iterations any box needed */
    int max_inner_used;     /* most FP32 V-cycles any box ran */
    int fallback_iters;     /* iterations run after the graph for boxes still above tolerance */
    int launches;           /* kernels launched by the step (graph nodes included) */
    int pad;
    double ms;              /* device time of the step (CUDA events) */
} nyxpm_ensemble_info;

nyxpm_status nyxpm_ensemble_create(nyxpm_ctx* ctx, size_t arena_bytes, nyxpm_ensemble** out);
nyxpm_status nyxpm_ensemble_destroy(nyxpm_ctx* ctx, nyxpm_ensemble* ens);
/* Device bytes one box of this shape takes from the arena. */
size_t nyxpm_ensemble_box_bytes(int n, int64_t np);
size_t nyxpm_ensemble_arena_used(const nyxpm_ensemble* ens);
/* Add a box (n >= 16, m * 2^k with m <= 8); NYXPM_OOM when the arena budget is exhausted. */
nyxpm_status nyxpm_ensemble_add(nyxpm_ctx* ctx, nyxpm_ensemble* ens, int n, double L, int64_t np,
                                int* slot);
nyxpm_status nyxpm_ensemble_remove(nyxpm_ctx* ctx, nyxpm_ensemble* ens, int slot);
/* Particles in (np x 3 positions and velocities, uniform mass); the box gets its
 * initial field at the a_old of its first step. */
nyxpm_status nyxpm_ensemble_upload(nyxpm_ctx* ctx, nyxpm_ensemble* ens, int slot, const double* pos,
                                   const double* vel, double mass);
nyxpm_status nyxpm_ensemble_download(nyxpm_ctx* ctx, nyxpm_ensemble* ens, int slot, double* pos,
                                     double* vel);
nyxpm_status nyxpm_ensemble_get_phi(nyxpm_ctx* ctx, nyxpm_ensemble* ens, int slot, double* phi);
/* The FP32 gravity vector the kicks use, widened to FP64 (3 n^3, component-major). */
nyxpm_status nyxpm_ensemble_grav_vector(nyxpm_ctx* ctx, nyxpm_ensemble* ens, int slot, double* g_out);
nyxpm_status nyxpm_ensemble_set_tuning(nyxpm_ctx* ctx, nyxpm_ensemble* ens, const nyxpm_tuning* t);
nyxpm_status nyxpm_ensemble_get_tuning(nyxpm_ctx* ctx, nyxpm_ensemble* ens, nyxpm_tuning* t);
/* One PM step (old-time field reused: kick-drift, deposit, solve, kick) of every
 * slot with a_old[slot] > 0; arrays are indexed by slot; other slots idle. */
nyxpm_status nyxpm_ensemble_step(nyxpm_ctx* ctx, nyxpm_ensemble* ens, const double* a_old,
                                 const double* a_new, const double* dt, nyxpm_ensemble_info* info);

/* ---- allocation-free deposit ----------------------------------------------------- */

/* The CIC mass density of np particles of equal mass that are already in device
 * memory (positions as three device arrays x, y, z in [0, L) up to one cell
 * outside), written to the caller's device array rho (n^3 doubles, x fastest),
 * on `stream` (a cudaStream_t; NULL is the default stream).  No counterpart in
 * the reference.  For callers that cannot allocate device memory themselves or
 * let a library do it -- a host code whose device memory is owned by its own
 * arena (an AMReX build reserves most of the GPU at start-up), where an extra
 * cudaMalloc can fail or fragment that arena.  This call allocates nothing: the
 * counting-sort scratch is a file-scope device array of about 10 MiB that every
 * GPU loading this library holds until the process exits.  Limits: n <= 64 and
 * np <= 262,144; larger problems return NYXPM_INVALID_ARG (use nyxpm_deposit).
 * Each call on a stream that is not capturing looks up the array's device
 * address on the current device (a device reset may move it); a call on a
 * capturing stream uses the address the last such call found, so make one call
 * on the device before any stream capture.  On a stream that is not capturing
 * the call returns once the stream has finished the deposit: it reads back a
 * count of non-finite positions, and refuses such input with NYXPM_INVALID_ARG
 * (rho then holds no valid density), as nyxpm_deposit does.  On a capturing
 * stream it only enqueues the deposit (a capture cannot be waited for): finite
 * positions at every replay are then the caller's to ensure.  All calls share the one array: calls that overlap on
 * the GPU (other streams, other host threads) race and must be ordered by the
 * caller.  The result equals nyxpm_deposit's for the same particles in the same
 * order, bit for bit.  errbuf (may be NULL) receives a message on failure. */
nyxpm_status nyxpm_deposit_noalloc(const double* x, const double* y, const double* z, int64_t np,
                                   double mass, int n, double L, double* rho, void* stream,
                                   char* errbuf, size_t errlen);

/* ---- multilevel (AMR) PM without subcycling, FP64 ------------------------------------
 * Nyx::advance_particles_only with finest_level > 0 and amr.subcycling_mode = None
 * (Source/TimeStep/Nyx_advance_particles.cpp:9-272) on fixed grids, as the
 * reference's Exec/ParticleOnlyTest/inputs.mass.nosub runs it (amr.regrid_file).
 * Level l has n0 * 2^l cells per side (refinement ratio 2); levels 1 .. nlev-1
 * (nlev <= 4) are lists of boxes given as 6 ints each (lo x y z, hi x y z,
 * inclusive, in that level's index space), level by level, nbox[l-1] on level l.
 * A box needs even lo and odd hi (coarsenable), boxes of a level must not
 * overlap, and each box above level 1 must sit inside the coarser level with
 * one coarse cell to spare.  A particle belongs to the finest level whose boxes
 * hold its cell.  The multilevel deposit (AMReX AssignDensity) and the composite
 * MLMG solve are AMReX's, absent from the reference tree; this library's
 * definition of both is given in nyx_gb300/csrc/pm_amr.cu. */
typedef struct nyxpm_amr nyxpm_amr;

nyxpm_status nyxpm_amr_create(nyxpm_ctx* ctx, int n0, double L, int nlev, const int* nbox,
                              const int* boxes, int64_t np, nyxpm_amr** out);
nyxpm_status nyxpm_amr_destroy(nyxpm_ctx* ctx, nyxpm_amr* amr);
/* pos, vel: np x 3; mass: np, or NULL with mass_scalar for equal masses.
 * mass_offset = sum(m) / L^3 (Gravity::set_mass_offset, Gravity.cpp:975-1030). */
nyxpm_status nyxpm_amr_upload(nyxpm_ctx* ctx, nyxpm_amr* amr, const double* pos,
                              const double* vel, const double* mass, double mass_scalar);
nyxpm_status nyxpm_amr_download(nyxpm_ctx* ctx, nyxpm_amr* amr, double* pos, double* vel);
/* One step: particle levels, old-time multilevel deposit and solve
 * (Gravity::multilevel_solve_for_old_phi, Gravity.cpp:572-600 ->
 * actual_multilevel_solve, :602-779), moveKickDrift on every level, new-time
 * deposit and solve (multilevel_solve_for_new_phi, :543-570), moveKick on every
 * level (DarkMatterParticleContainer.cpp:76-247), the periodic shift of
 * post_timestep (Nyx.cpp:1421-1437).  Both solves start from phi = 0, as the
 * reference calls them (use_previous_phi_as_guess defaults to 0, Gravity.H:64-69).
 * NYXPM_INVALID_ARG if a particle moved more than 2 cells of its level. */
nyxpm_status nyxpm_amr_step(nyxpm_ctx* ctx, nyxpm_amr* amr, double a_old, double a_new,
                            double dt, nyxpm_step_info* info);
/* The parts of the step, for callers that drive it themselves:
 * particle levels and boxes (box -1 on level 0) of the current positions; */
nyxpm_status nyxpm_amr_assign(nyxpm_ctx* ctx, nyxpm_amr* amr, int* lev, int* box);
/* multilevel CIC deposit with the levels of the last nyxpm_amr_assign
 * (Gravity::AddParticlesToRhs, Gravity.cpp:1068-1102); */
nyxpm_status nyxpm_amr_deposit(nyxpm_ctx* ctx, nyxpm_amr* amr);
/* composite solve of the deposited density at a, from phi = 0; */
nyxpm_status nyxpm_amr_solve(nyxpm_ctx* ctx, nyxpm_amr* amr, double a, nyxpm_solve_info* info);
/* gravity vector of every level (Gravity::get_old_grav_vector / get_new_grav_vector); */
nyxpm_status nyxpm_amr_grav_vector(nyxpm_ctx* ctx, nyxpm_amr* amr);
/* kick (and drift when do_move) of every particle with its own level's g. */
nyxpm_status nyxpm_amr_kick(nyxpm_ctx* ctx, nyxpm_amr* amr, double dt, double a_prev,
                            double a_cur, int do_move);
/* A field of level 0 (box -1: n0^3, x fastest) or of one box (its cells, x
 * fastest); which: NYXPM_AMR_RHO .. NYXPM_AMR_MASS. */
enum { NYXPM_AMR_RHO = 0, NYXPM_AMR_PHI = 1, NYXPM_AMR_GX = 2, NYXPM_AMR_GY = 3, NYXPM_AMR_GZ = 4,
       NYXPM_AMR_MASS = 5 };
nyxpm_status nyxpm_amr_field(nyxpm_ctx* ctx, nyxpm_amr* amr, int which, int box, double* out);
/* Cells of level 0 (box -1) or of one box; -1 for a bad box. */
int64_t nyxpm_amr_cells(const nyxpm_amr* amr, int box);

/* ---- measurement ------------------------------------------------------------- */

#define NYXPM_NUM_STAGES 12
/* Stage ids of nyxpm_profile. */
enum {
    NYXPM_ST_KEYS = 0, NYXPM_ST_SCAN, NYXPM_ST_SCATTER, NYXPM_ST_GATHER, NYXPM_ST_DEPOSIT,
    NYXPM_ST_RHS, NYXPM_ST_SMOOTH, NYXPM_ST_RESTRICT, NYXPM_ST_PROLONG, NYXPM_ST_BOTTOM,
    NYXPM_ST_NORM, NYXPM_ST_KICK
};

typedef struct nyxpm_profile {
    int64_t launches[NYXPM_NUM_STAGES];
    double ms[NYXPM_NUM_STAGES];          /* summed CUDA-event time per stage */
    double bytes[NYXPM_NUM_STAGES];       /* summed algorithmic bytes per stage */
    /* finest-level red-black half sweeps only (the dominant kernel) */
    int64_t fine_smooth_launches;
    double fine_smooth_ms;
    double fine_smooth_bytes;
} nyxpm_profile;

/* Record a CUDA event pair around every launch (off by default). */
nyxpm_status nyxpm_set_profiling(nyxpm_ctx* ctx, int on);
/* Synchronises, folds the recorded events into *out (accumulated since the last
 * reset) and optionally resets. */
nyxpm_status nyxpm_get_profile(nyxpm_ctx* ctx, nyxpm_profile* out, int reset);
/* Number of kernels the context launched since creation. */
int64_t nyxpm_launch_count(const nyxpm_ctx* ctx);
/* The FP64 rate this GPU sustains, in TFLOP/s (a fused multiply-add counts as two
 * operations): chains of dependent FP64 FMAs filling every SM, timed with CUDA
 * events on the context's stream (the best over four launch shapes of three runs
 * of about 10 ms, each shape after one warm-up run); add_tops (may be NULL)
 * receives the rate of FP64 additions measured the same way, in T additions/s.
 * The denominators of the FP64 roofline of the FP64 form, whose kernels are bound
 * by the FP64 pipe.  No counterpart in the reference. */
nyxpm_status nyxpm_measure_fp64_peak(nyxpm_ctx* ctx, double* tflops, double* add_tops);

#ifdef __cplusplus
}
#endif

#endif /* NYXPM_H */
