/* kmpm.h -- C ABI of the GB300-native explicit MPM time step (libkmpm.so).
 *
 * This is the boundary a Karamelo method style calls.  A maintainer adds the
 * styles `tlmpm/gpu` and `ulmpm/gpu` (Method, src/method.h:25-54, registered
 * through src/style_method.h) and `usl/gpu` / `musl/gpu` (Scheme,
 * src/scheme.h:19-24); their code uploads the state that Karamelo's host
 * classes built (Domain, Grid::init, Solid::populate, Material, Group, Fix)
 * and then lets kmpm_run() execute whole time steps on the GPU.
 *
 * Conventions
 *   - every function returns an int status: KMPM_OK (0) or a negative
 *     KMPM_ERR_* code; kmpm_last_error() gives the message.  The reference's
 *     fatal checks (Error::one / Error::all, src/error.cpp:33-68) come back as
 *     the KMPM_ERR_* codes of the step that raised them;
 *   - vectors are passed as arrays of n*3 doubles (the memory layout of
 *     std::vector<Eigen::Vector3d>), tensors as n*9 doubles in row-major
 *     order; particle arrays are in the order the caller uploaded them;
 *   - the context owns all device memory and one CUDA stream; host buffers
 *     stay owned by the caller; no call allocates device memory once
 *     kmpm_run() has started, except the first kmpm_run() after a solid or
 *     fix was added;
 *   - one host thread per context (the reference is single-threaded per rank).
 */
#ifndef KMPM_H
#define KMPM_H

#ifdef __cplusplus
extern "C" {
#endif

#define KMPM_OK 0
#define KMPM_ERR_ARG (-1)          /* bad argument or unsupported combination */
#define KMPM_ERR_CUDA (-2)         /* CUDA runtime failure / no device */
#define KMPM_ERR_STATE (-3)        /* call out of order */
#define KMPM_ERR_J (-10)           /* J <= 0, src/solid.cpp:1208-1215 */
#define KMPM_ERR_LEFT_DOMAIN (-11) /* particle left the box, src/solid.cpp:617-627 */
#define KMPM_ERR_NAN (-12)         /* nan wave speed / dtCFL, src/solid.cpp:1387-1397, src/tlmpm.cpp:498-508 */
#define KMPM_ERR_POLDEC (-13)      /* polar decomposition failed, src/solid.cpp:1229-1236 */
#define KMPM_ERR_DTCFL (-14)       /* dtCFL == 0, src/tlmpm.cpp:498-502 */
#define KMPM_ERR_TIMEOUT (-15)     /* a bounded wait inside a kernel ran out (tensor-core network, staged state rows) */

/* method / scheme / basis (Update::create_method, src/update.cpp:108-196) */
#define KMPM_TLMPM 0
#define KMPM_ULMPM 1
#define KMPM_USL 0
#define KMPM_MUSL 1
#define KMPM_USF 2       /* USF::run, src/usf.cpp:34-95 (FLIP/PIC transfers, mechanical runs) */
#define KMPM_BASIS_LINEAR 0
#define KMPM_BASIS_CUBIC 1
#define KMPM_BASIS_BERNSTEIN 2
#define KMPM_BASIS_QUADRATIC 3  /* quadratic B-spline, src/basis_functions.h:140-241 */

/* kmpm_params.transfer: the method's sub-type (Update::create_method,
 * src/update.cpp:129-149) */
#define KMPM_TRANSFER_FLIP 0
#define KMPM_TRANSFER_APIC 1
#define KMPM_TRANSFER_AFLIP 2   /* ULMPM: affine transfers with the FLIP blend; TLMPM: as FLIP */
#define KMPM_TRANSFER_ASFLIP 3  /* AFLIP with positions moved by the blended velocity (ULMPM) */
#define KMPM_TRANSFER_MLS 4     /* ULMPM only: APIC with internal forces from moments */

/* kmpm_params.precision: arithmetic of the three places that the FP32 bulk
 * may promote (nodal v = p/m, det/inverse of F, the constitutive return) */
#define KMPM_PREC_FP32 0
#define KMPM_PREC_FP64_ISLANDS 1

typedef struct {
  int method;        /* KMPM_TLMPM / KMPM_ULMPM */
  int scheme;        /* KMPM_USL / KMPM_MUSL / KMPM_USF (src/update.cpp:42-45 default MUSL) */
  int basis;         /* KMPM_BASIS_* */
  int dim;           /* 1, 2 or 3 (Domain::dimension) */
  double pic_flip;   /* Update::PIC_FLIP (0 for PIC) */
  int thermal;       /* method(..., thermo-mechanical) */
  double dt;         /* Update::dt at the first step (1e-16 unless set_dt) */
  double dt_factor;  /* Update::dt_factor */
  int dt_constant;   /* set_dt() was used */
  double boxlo[3];   /* Domain::boxlo / boxhi */
  double boxhi[3];
  int precision;     /* KMPM_PREC_* */
  int track_strain;  /* keep Solid::strain_el (needed by the strain-energy output) */
  int independent;   /* TLMPM only: every solid is an independent simulation with its own
                        dt and time (a batch of runs in one launch per phase); 0 = one
                        simulation whose dt is the minimum over solids (adjust_dt) */
  int autotune;      /* 1: at the first kmpm_run / kmpm_run_time after at least one step,
                        time every launch shape of the gather kernels on a scratch copy of
                        the particle state and keep the fastest (kmpm_tuning reports it) */
  int transfer;      /* KMPM_TRANSFER_*: the method's sub-type.  FLIP: PIC/FLIP blend by pic_flip.
                        APIC (and for ULMPM AFLIP, ASFLIP, MLS): affine transfers,
                        src/solid.cpp:392-426, 524-574, 1006-1153; cubic or quadratic spline,
                        mechanical runs; APIC and MLS set pic_flip = 0 */
  int axisymmetric;  /* Domain::axisymmetric (src/domain.cpp:554-570): 2-D runs with x = r and
                        y = z.  Adds the hoop terms: -vol0 PK1(2,2) w / x0_r (TL) or
                        -vol sigma(2,2) w / x_r (UL) to the radial node force
                        (src/solid.cpp:472-475, 513-519, 565-571) and v_r w / r to
                        Fdot(2,2) / L(2,2) (src/solid.cpp:818-829, 900-913, 1046-1058,
                        1120-1132).  The caller passes masses and volumes already
                        multiplied by x0_r (Solid::populate, src/solid.cpp:2292-2295).
                        Mechanical runs only (src/solid.cpp:2789-2792). */
} kmpm_params;

/* One material: Mat (src/material.h:45-68) with its EOS / Strength / Damage /
 * Temperature parameters in the argument order of the reference commands:
 *   eos_p   linear (rho0,K); shock (rho0,K,c0,S,Gamma,cv,Tr,Q1,Q2); fluid (rho0,K,Gamma)
 *   str_p   linear (G); plastic (G,sigmay); johnson_cook (G,A,B,n,epsdot0,C,m,Tr,Tm);
 *           swift (G,A,B,C,n); fluid (mu)
 *   dam_p   damage_johnson_cook (d1,d2,d3,d4,d5,epsdot0,Tr,Tm)
 *   temp_p  plastic_work (chi,cp,kappa,alpha,T0,Tm) */
#define KMPM_MAT_LINEAR 0
#define KMPM_MAT_NEO_HOOKEAN 1
#define KMPM_MAT_EOS_STRENGTH 2
typedef struct {
  int type;
  double rho0, E, nu, cp, kappa; /* linear / neo-Hookean materials */
  int eos;                       /* 0 linear, 1 shock, 2 fluid */
  double eos_p[12];
  int strength;                  /* 0 linear, 1 plastic, 2 johnson_cook, 3 swift, 4 fluid */
  double str_p[12];
  int damage;                    /* -1 none, 0 damage_johnson_cook */
  double dam_p[8];
  int temp;                      /* -1 none, 0 plastic_work */
  double temp_p[6];
} kmpm_material;

/* fix kinds lowered to the device */
#define KMPM_FIX_VELOCITY_NODES 0 /* FixVelocityNodes, src/fix_velocity_nodes.cpp:130-271 */
#define KMPM_FIX_BODY_FORCE 1     /* FixBodyforce, src/fix_body_force.cpp:106-179 */

/* particle fields for kmpm_download_particles / kmpm_upload_particles */
#define KMPM_P_X 0        /* n*3 */
#define KMPM_P_X0 1       /* n*3 */
#define KMPM_P_V 2        /* n*3 */
#define KMPM_P_SIGMA 3    /* n*9, as stored (unrotated for TLMPM) */
#define KMPM_P_SIGMA_ROT 4 /* n*9, R sigma R^T for TLMPM dumps (src/dump_particle.cpp:98-102) */
#define KMPM_P_F 5        /* n*9 */
#define KMPM_P_EPS_P 6
#define KMPM_P_EPSDOT_P 7
#define KMPM_P_DAMAGE 8
#define KMPM_P_DAMAGE_INIT 9
#define KMPM_P_T 10
#define KMPM_P_J 11
#define KMPM_P_VOL 12
#define KMPM_P_STRAIN_EL 13 /* n*9 (needs kmpm_params.track_strain) */
#define KMPM_P_VOL0PK1 14 /* n*9, TLMPM: vol0 times the first Piola-Kirchhoff stress of the last stress update */
#define KMPM_P_MASS 15
#define KMPM_P_SIGMA_ROT6 16 /* n*6: the rotated stress as the reference dump writes it,
                                s11 s22 s33 s12 s13 s23 (src/dump_particle.cpp:116-121); download only */

/* grid fields for kmpm_download_grid */
#define KMPM_G_MASS 0
#define KMPM_G_V 1
#define KMPM_G_V_UPDATE 2
#define KMPM_G_X 3
#define KMPM_G_T 6

/* Context life cycle.  Replaces what Update::create_method / Method::setup
 * (src/update.cpp:108-196, src/tlmpm.cpp:51-85) configure. */
int kmpm_create(const kmpm_params *params, struct kmpm_ctx **out);
int kmpm_destroy(struct kmpm_ctx *ctx);
const char *kmpm_last_error(const struct kmpm_ctx *ctx);

/* Material::add_material (src/material.cpp:249-380); returns the id (>= 0). */
int kmpm_add_material(struct kmpm_ctx *ctx, const kmpm_material *mat);

/* Grid::init (src/grid.cpp:68-413): the caller passes the node lattice it
 * built (lower bound, cellsize, local node counts n[3] and global counts
 * nglobal[3] used by the boundary-modified cubic splines).  Returns the id. */
int kmpm_add_grid(struct kmpm_ctx *ctx, const double lo[3], double cellsize, const int n[3], const int nglobal[3]);

/* Solid state after Solid::populate (src/solid.cpp:1810-2336): n particles
 * with x0, x, v (n*3), mass, vol0 (n) and the initial temperature.  TLMPM
 * solids each own one grid; ULMPM solids share grid 0.  Returns the id. */
int kmpm_add_solid(struct kmpm_ctx *ctx, int grid, int mat, int n, const double *x0, const double *x,
                   const double *v, const double *mass, const double *vol0, double T0);

/* Solid::np_per_cell, the particles per cell per direction the solid was
 * populated with (src/solid.cpp:2027).  Needed only by APIC with the linear
 * basis, whose inertia tensor depends on it (1 or 2, src/solid.cpp:1447-1462). */
int kmpm_set_np_per_cell(struct kmpm_ctx *ctx, int solid, int np_per_cell);

/* A fix on the nodes of one grid.  coef[4*d..4*d+3] = (c0,c1,c2,c3) give the
 * value of axis d as c0 + c1*time + c2*exp(c3*time) (velocity_nodes) or the
 * constant acceleration c0 (body_force); set[d] != 0 selects the axes. */
int kmpm_add_fix(struct kmpm_ctx *ctx, int kind, int grid, const unsigned char *node_mask, const int set[3],
                 const double coef[12]);

/* Contact fixes between two solids, evaluated at the start of every step
 * (Modify::initial_integrate): each particle pair closer than Rp1 + Rp2
 * (Rp = half the cube root of the current volume in 3-D, half its square
 * root in 2-D) adds equal and opposite forces to the external force vector
 * mbp of its two particles, which the scatter then adds to the node forces.
 * Pairs are found on a hashed cell list of the current positions with the
 * larger of the two grids' cellsizes as its cell; each particle sums its
 * own pairs, so the result does not depend on scheduling.
 *   KMPM_CONTACT_MIN_PENETRATION: FixContactMinPenetration::initial_integrate
 *     (src/fix_contact_min_penetration.cpp:83-235), with Coulomb friction mu
 *     and, in thermo-mechanical runs, frictional heating;
 *   KMPM_CONTACT_HERTZ: FixContactHertz::initial_integrate
 *     (src/fix_contact_hertz.cpp:82-197); mu is ignored.
 * Both solids must differ; independent batches take no contact.  Returns the
 * contact's id (>= 0). */
#define KMPM_CONTACT_MIN_PENETRATION 0
#define KMPM_CONTACT_HERTZ 1
int kmpm_add_contact(struct kmpm_ctx *ctx, int kind, int solid1, int solid2, double mu);

/* Total contact force of the last step (the variables <id>_x, <id>_y, <id>_z
 * the reference fix sets): the sum over all pairs of the force on solid1
 * (min-penetration) or on solid2 (Hertz).  Zero before the first step. */
int kmpm_contact_force(struct kmpm_ctx *ctx, int contact, double out[3]);

/* Scheme::run for nsteps steps (USL::run src/usl.cpp:34-94, MUSL::run
 * src/musl.cpp:34-95), each step fully on the GPU. */
int kmpm_run(struct kmpm_ctx *ctx, int nsteps);

/* kmpm_run without the wait (no counterpart in the reference, whose steps
 * run on the calling thread): the nsteps steps are queued on the context's
 * stream and the call returns, so that the caller can queue downloads and
 * further runs while the GPU steps.  A step's error (J <= 0, a particle
 * outside the domain, ...) does not stop the steps queued after it, as
 * within one kmpm_run; the next kmpm_sync or kmpm_run reports the first one,
 * with its step.  Calls that read the device state (kmpm_scalars, the
 * downloads) run in order after the queued steps. */
int kmpm_run_async(struct kmpm_ctx *ctx, int nsteps);

/* Wait for every step queued on the context's stream and report the first
 * error any of them raised (KMPM_OK if none). */
int kmpm_sync(struct kmpm_ctx *ctx);

/* RunTime::command (src/run_time.cpp:30-60): steps until time >= maxtime. */
int kmpm_run_time(struct kmpm_ctx *ctx, double maxtime, int *nsteps_done);

/* At most nsteps steps of a RunTime::command (src/run_time.cpp:30-60): stops
 * once time >= maxtime, so that a caller can end a run_time at its output
 * steps (Output::next) as the reference's scheme loop does
 * (src/musl.cpp:82-91).  nsteps_done (may be NULL) receives the steps run. */
int kmpm_run_until(struct kmpm_ctx *ctx, int nsteps, double maxtime, int *nsteps_done);

/* Update::atime, Update::dt, Update::ntimestep. */
int kmpm_scalars(struct kmpm_ctx *ctx, double *time, double *dt, long long *ntimestep);

/* The same for one solid of an independent batch (kmpm_params.independent). */
int kmpm_solid_scalars(struct kmpm_ctx *ctx, int solid, double *time, double *dt, long long *ntimestep);

/* Download / upload one particle field of one solid in the caller's
 * particle order (the download before Output::write, src/output.cpp:128-200). */
int kmpm_download_particles(struct kmpm_ctx *ctx, int solid, int field, double *out);

/* Upload one particle field of one solid (caller order, the layout of
 * kmpm_download_particles).  Before the first run: KMPM_P_X, KMPM_P_X0 and
 * KMPM_P_V (the arrays kmpm_add_solid took).  After it (kmpm_run(ctx, 0)
 * builds the context): KMPM_P_X, KMPM_P_V, KMPM_P_SIGMA (as stored: the
 * corotational frame for TLMPM), KMPM_P_F, KMPM_P_EPS_P, KMPM_P_EPSDOT_P,
 * KMPM_P_DAMAGE, KMPM_P_DAMAGE_INIT, KMPM_P_T, KMPM_P_STRAIN_EL and, for
 * TLMPM, KMPM_P_VOL0PK1 -- the particle state Solid::read_restart restores
 * (src/solid.cpp:2894-2957); L, Fdot and the APIC matrix restart at zero, as
 * there.  The device keeps positions as x0 + u and F as I + H (FP32 u, H):
 * x and F pass through FP64 sums, exact unless u or H is more than 2^29
 * times smaller than x0 or 1, where their last bits go (kmpm_save_state
 * keeps them). */
int kmpm_upload_particles(struct kmpm_ctx *ctx, int solid, int field, const double *in);

/* Update::atime, Update::dt and Update::ntimestep as a restart sets them
 * (Update::read_restart, src/update.cpp:303-338); every solid of an
 * independent batch gets the same values. */
int kmpm_set_scalars(struct kmpm_ctx *ctx, double time, double dt, long long ntimestep);

/* Device snapshot (no counterpart in the reference, which restarts from the
 * host state above): the particle buffer in its binned slot order, the step
 * scalars and the node arrays, copied raw.  kmpm_load_state on a context made
 * by the same setup calls restores the state bit for bit, so that the run
 * continues exactly as if it had not stopped.  kmpm_state_size gives the
 * bytes kmpm_save_state writes. */
int kmpm_state_size(struct kmpm_ctx *ctx, unsigned long long *bytes);
int kmpm_save_state(struct kmpm_ctx *ctx, void *out, unsigned long long bytes);
int kmpm_load_state(struct kmpm_ctx *ctx, const void *in, unsigned long long bytes);

/* Asynchronous download (no counterpart in the reference, whose dumps stop
 * the run while they write): the field is gathered on the context's stream in
 * order with the steps, then copied to `out` on a second stream while later
 * kmpm_run calls proceed.  `out` must be page-locked host memory
 * (cudaHostAlloc / cudaHostRegister) of n*width doubles and stays owned by
 * the caller; its content is valid after kmpm_sync_downloads (every queued
 * download) or kmpm_wait_download(ctx, out) (the last one queued into `out`,
 * leaving later downloads in flight; KMPM_OK at once if none is). */
int kmpm_download_particles_async(struct kmpm_ctx *ctx, int solid, int field, double *out);
int kmpm_sync_downloads(struct kmpm_ctx *ctx);
int kmpm_wait_download(struct kmpm_ctx *ctx, const double *out);

/* Download one grid field (n*1 or n*3 doubles, reference node order). */
int kmpm_download_grid(struct kmpm_ctx *ctx, int grid, int field, double *out);

/* out[0] = kinetic energy (FixKineticEnergy, src/fix_kinetic_energy.cpp:78-118),
 * out[1] = strain energy (ComputeStrainEnergy, src/compute_strain_energy.cpp:64-117),
 * both over all solids, reduced on the device in a fixed order. */
int kmpm_energy(struct kmpm_ctx *ctx, double out[2]);

/* The context's CUDA stream (cudaStream_t as void*), for callers that time or
 * order their own work around kmpm_run. */
void *kmpm_stream(struct kmpm_ctx *ctx);

/* Number of kernel launches one time step issues (for launch accounting). */
int kmpm_launches_per_step(struct kmpm_ctx *ctx);

/* The autotuner's record (no counterpart in the reference): a JSON object
 * with the candidate launch shapes of each gather kernel, their times in ms
 * and the one chosen; "{}" before tuning. */
const char *kmpm_tuning(struct kmpm_ctx *ctx);

/* Profiling (no counterpart in the reference): runs nsteps steps launched
 * eagerly with a CUDA event recorded on the context's stream after every
 * phase, and returns the mean device time of each phase in phase_ms (at most
 * max_phases); kmpm_profile_phase() names phase i ("p2g", "grid_update",
 * "g2p_advance", "p2g_velocity", "grid_velocity", "g2p_stress", "dt", ...). */
int kmpm_profile(struct kmpm_ctx *ctx, int nsteps, double *phase_ms, int max_phases, int *nphases);
const char *kmpm_profile_phase(struct kmpm_ctx *ctx, int i);

/* ------------------------------------------------------------------------
 * Learned Johnson-Cook return map.  No counterpart in the reference, which
 * evaluates StrengthJohnsonCook::update_deviatoric_stress
 * (src/strength_jc.cpp:100-184) in closed form.
 *
 * The network is an MLP 15 -> 128 -> 128 -> 128 -> 7 with ReLU hidden layers.
 *   inputs  (KMPM_MLP_NIN): strain increment dt*D (6: xx yy zz xy xz yz, in the
 *           corotational frame), Cauchy stress before the step (6), equivalent
 *           plastic strain, temperature, log(1 + epsdot_p / epsdot0)
 *   outputs (KMPM_MLP_NOUT): s_new - s_trial (6), plastic strain increment
 * It is trained on the GPU in FP32 (kmpm_mlp_train) and evaluated as BF16
 * tensor-core MMAs with FP32 accumulation (kmpm_set_surrogate): over the
 * plastic steps the G2P stress kernel queues when every material is linear
 * EOS + Johnson-Cook, else inside that kernel.  Parameters are one flat FP32 vector of
 * KMPM_MLP_NPARAMS values: W1[128x15] b1[128] W2[128x128] b2 W3[128x128] b3
 * W4[7x128] b4[7] (row-major, out x in).  The normalisation vector holds
 * in_mean[15] in_std[15] out_mean[7] out_scale[7] env_lo[15] env_hi[15];
 * the envelope bounds are in normalised units.  Arrays named X and Y in the
 * kmpm_mlp_* calls are DEVICE pointers, row-major, in physical units. */
#define KMPM_MLP_NIN 15
#define KMPM_MLP_NOUT 7
#define KMPM_MLP_NPARAMS 35975
#define KMPM_MLP_NNORM 74
struct kmpm_mlp;
typedef struct {
  int batch;              /* rows per step, <= the batch given to kmpm_mlp_create */
  long long steps;        /* optimiser steps (Adam, beta 0.9 / 0.999) */
  double lr;              /* initial learning rate, cosine decay to lr * lr_final_ratio */
  double lr_final_ratio;
  unsigned long long seed;  /* batches are drawn with replacement by a hash of (seed, step, row) */
  int report_every;       /* print the batch loss to stderr every this many steps (0: never) */
} kmpm_train_opts;
int kmpm_mlp_create(int batch, struct kmpm_mlp **out);
void kmpm_mlp_destroy(struct kmpm_mlp *m);
const char *kmpm_mlp_last_error(const struct kmpm_mlp *m);
/* He-uniform weights from a seeded splitmix64 stream, zero biases, fresh optimiser state. */
int kmpm_mlp_init(struct kmpm_mlp *m, unsigned long long seed);
int kmpm_mlp_set_params(struct kmpm_mlp *m, const float *params);  /* host array */
int kmpm_mlp_get_params(struct kmpm_mlp *m, float *params);
int kmpm_mlp_set_norm(struct kmpm_mlp *m, const float *norm);      /* host array */
int kmpm_mlp_get_norm(struct kmpm_mlp *m, float *norm);
/* Mean squared error over n rows in normalised output units and its gradient
 * (host outputs; grad has KMPM_MLP_NPARAMS values). */
int kmpm_mlp_loss_grad(struct kmpm_mlp *m, const float *X, const float *Y, int n, float *loss, float *grad);
int kmpm_mlp_train(struct kmpm_mlp *m, const float *X, const float *Y, long long n, const kmpm_train_opts *opts,
                   float *final_loss);
/* FP32 inference (the training kernels) and tensor-core inference (BF16
 * operands, FP32 accumulation: the arithmetic of the learned G2P kernel);
 * inside (may be NULL) receives 1 where every input lies in the envelope. */
int kmpm_mlp_predict(struct kmpm_mlp *m, const float *X, long long n, float *Y);
int kmpm_mlp_predict_tc(struct kmpm_mlp *m, const float *X, long long n, float *Y, signed char *inside);

/* Training pairs from the plain GPU path: while logging is on, the stress
 * kernel writes (15 inputs, 7 outputs) of a hashed fraction of the plastic
 * particle-steps (undamaged Johnson-Cook particles) into a device buffer of
 * capacity rows; kmpm_log_data returns its device address and the number of
 * rows written.  TLMPM, 3-D, cubic B-spline, FP32, eos-strength materials
 * with Johnson-Cook strength only (KMPM_ERR_ARG otherwise). */
int kmpm_log_start(struct kmpm_ctx *ctx, long long capacity, double fraction, unsigned long long seed);
int kmpm_log_stop(struct kmpm_ctx *ctx);
int kmpm_log_data(struct kmpm_ctx *ctx, const float **rows, long long *n);
/* Closed-form return map of one material on n input rows (device arrays):
 * Y has 8 columns, the 7 outputs and a plastic flag (1 or 0). */
int kmpm_jc_label(struct kmpm_ctx *ctx, int material, const float *X, long long n, float *Y);
/* Replace the closed-form return map on plastic steps by the network (a copy
 * of its current parameters is taken).  The predicted stress correction is
 * kept through its component along the trial deviator (J2 flow is radial).
 * A network answer is used only where every input lies in the envelope and
 * its yield-function residual |s_eq(new) - flow stress| and flow-rule
 * residual |s_eq(trial) - s_eq(new) - 3 G dep| are both <= tol times the flow
 * stress; the closed form is used everywhere else.  m == NULL restores the
 * plain path.  Same restrictions as kmpm_log_start. */
int kmpm_set_surrogate(struct kmpm_ctx *ctx, struct kmpm_mlp *m, double tol);
/* Particle-steps since kmpm_set_surrogate: out[0] plastic, out[1] served by
 * the network, out[2] outside the envelope, out[3] residual above tol. */
int kmpm_surrogate_stats(struct kmpm_ctx *ctx, long long out[4]);

/* Nodal mass without device allocation.  No counterpart in the reference.
 *
 * For host applications that own all of their GPU memory through their own
 * pool allocator and budget: they reserve the device memory up front and may
 * not call cudaMalloc behind the pool's back (the call could fail once the
 * pool holds the memory, and it would escape their accounting).  The caller
 * passes device buffers: x (n*3 floats, x y z per particle), mass (n floats)
 * and node_mass (one float per node of the grid described by lo, cellsize,
 * nnodes and nglobal, as in kmpm_add_grid; basis 0-3 as KMPM_BASIS_*); the
 * result is what Solid::compute_mass_nodes (src/solid.cpp:317-335) computes,
 * by the same deterministic scatter that kmpm_run uses, bit for bit.  Nothing
 * is allocated: every intermediate array lives in one fixed-size device array
 * of KMPM_NOALLOC_SCRATCH_BYTES that every GPU loading this library holds
 * until the process exits.  Limits: at most KMPM_NOALLOC_MAX_PARTICLES
 * particles and KMPM_NOALLOC_MAX_CELLS binning cells (larger problems return
 * KMPM_ERR_ARG with a message in err).  A particle outside the grid's cells
 * (or with a non-finite coordinate) makes the call return
 * KMPM_ERR_LEFT_DOMAIN, and node_mass is then not meaningful.  Work is queued
 * on `stream` (a cudaStream_t, may be 0), and the call returns once that work
 * has finished, because the status depends on it.  The first call on a device
 * looks up that array's device address: make it before any stream capture.
 * Calls share the array; two calls that overlap on the GPU race on it.  err
 * (errlen bytes, may be NULL) receives the message of a failure. */
#define KMPM_NOALLOC_MAX_PARTICLES 131072
#define KMPM_NOALLOC_MAX_CELLS 262144
#define KMPM_NOALLOC_SCRATCH_BYTES (24u << 20)
int kmpm_p2g_mass_noalloc(const float *x, const float *mass, int n, int dim, int basis, const double lo[3],
                          double cellsize, const int nnodes[3], const int nglobal[3], float *node_mass, void *stream,
                          char *err, int errlen);

#ifdef __cplusplus
}
#endif
#endif /* KMPM_H */
