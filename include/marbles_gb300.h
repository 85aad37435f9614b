/* marbles_gb300.h -- C ABI of the GB300-native MARBLES level step.
 *
 * One opaque context owns every device buffer of one simulation (all AMR
 * levels).  Calls on a context are serialised on its CUDA stream; a context is
 * not re-entrant.  No call aborts or throws: each returns an mbg_status and
 * mbg_last_error() gives the message of the last failure.
 *
 * Host arrays of per-cell data use the layout of an AMReX FArrayBox without
 * ghost cells, concatenated over the boxes of the level in the order they
 * were defined:   [box][component][k][j][i]   (i fastest).
 *
 * Reference interfaces (paths inside the NREL/marbles project) that these
 * entry points replace are cited on each declaration.
 */
#ifndef MARBLES_GB300_H
#define MARBLES_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mbg_ctx mbg_ctx;

typedef enum {
    MBG_OK = 0,
    MBG_EINVAL = 1,      /* bad argument or unsupported configuration        */
    MBG_ENOMEM = 2,      /* device allocation failed                         */
    MBG_ECUDA = 3,       /* a CUDA call failed                               */
    MBG_ETIMEOUT = 4,    /* a bounded device-side wait ran out               */
    MBG_ESTATE = 5       /* call out of order (e.g. level not defined)       */
} mbg_status;

/* storage / arithmetic forms of the populations */
typedef enum {
    MBG_FP64 = 0,          /* FP64 storage and arithmetic (the reference's)   */
    MBG_FP32C_F16S = 1,    /* FP16 shifted storage, FP32 arithmetic           */
    MBG_FP32C_BF16S = 2    /* BF16 shifted storage, FP32 arithmetic           */
} mbg_precision;

/* boundary-condition codes of lbm.bc_lo / lbm.bc_hi (Source/BC.H:13-20) */
enum {
    MBG_BC_PERIODIC = 0, MBG_BC_NOSLIP = 1, MBG_BC_VELOCITY = 2,
    MBG_BC_PRESSURE = 3, MBG_BC_OUTFLOW = 5, MBG_BC_SLIPX = 6,
    MBG_BC_SLIPY = 7, MBG_BC_SLIPZ = 8
};

/* lbm.velocity_bc_type (Source/VelocityBC.H:13-199) */
enum { MBG_VBC_NOOP = 0, MBG_VBC_CONSTANT = 1, MBG_VBC_CHANNEL = 2, MBG_VBC_PARABOLIC = 3 };

/* Per-simulation parameters.  Each field is the inputs key named beside it
 * (Source/LBM.cpp:196-300, Source/VelocityBC.cpp:4-57). */
typedef struct mbg_params {
    int n_cell[3];               /* amr.n_cell (level 0)                       */
    double prob_lo[3];           /* geometry.prob_lo                           */
    double prob_hi[3];           /* geometry.prob_hi                           */
    int is_periodic[3];          /* geometry.is_periodic                       */
    int bc_lo[3], bc_hi[3];      /* lbm.bc_lo, lbm.bc_hi                        */
    double nu;                   /* lbm.nu                                     */
    double alpha;                /* lbm.alpha (defaults to nu)                 */
    double dx_outer, dt_outer;   /* lbm.dx_outer, lbm.dt_outer                 */
    double adiabatic_exponent;   /* lbm.adiabatic_exponent                     */
    double m_bar;                /* lbm.mean_molecular_mass                    */
    int precision;               /* mbg_precision                              */
    /* reference state of the shifted 16-bit storage (ignored for FP64):
     * populations are stored as (f - f_rest) / scale, f_rest the equilibrium
     * at (rho_ref, u = 0, T_ref) */
    double rho_ref, t_ref;
    /* velocity BC functor (lbm.velocity_bc_type, velocity_bc_<type>.*) */
    int velbc_type;
    int vbc_dir;                 /* velocity_bc_constant.dir                   */
    int vbc_normal_dir;          /* velocity_bc_parabolic.normal_dir           */
    int vbc_tangential_dir;      /* velocity_bc_parabolic.tangential_dir       */
    double vbc_u_ref;            /* Mach_ref * speed_of_sound_ref              */
    double vbc_initial_density;
    double vbc_initial_temperature;
    double vbc_adiabatic_exponent;
    double vbc_m_bar;
    /* reference velocity of the shifted 16-bit storage: the rest state above
     * is taken at (rho_ref, u_ref, T_ref), e.g. the inflow velocity of a
     * channel flow, so that the stored deviations carry the perturbation only */
    double u_ref[3];
} mbg_params;

/* Create a context on the current CUDA device.  cuda_stream may be NULL (the
 * context then creates its own stream).  Replaces the construction of the
 * LBM object's level data (Source/LBM.cpp:6-151, LBM.H:25-319). */
mbg_status mbg_create(const mbg_params* params, void* cuda_stream, mbg_ctx** out);

/* Release every device buffer of the context. */
void mbg_destroy(mbg_ctx* ctx);

/* Message of the last failed call on this context (or of the last failed
 * mbg_create when ctx is NULL). */
const char* mbg_last_error(const mbg_ctx* ctx);

/* Define level lev (0 = coarsest; ratio 2 between levels) from nbox boxes,
 * lohi[6*n .. 6*n+5] = lo_x lo_y lo_z hi_x hi_y hi_z (inclusive, in the
 * level's index space), and the is_fluid flags of each box grown by 3 ghost
 * cells: flags[off_n + ((k+3)*(ny+6) + (j+3))*(nx+6) + (i+3)], bit 0 =
 * is_fluid component 0, bit 1 = component 1 (eb_boundary), where off_n is the
 * running sum of (nx+6)(ny+6)(nz+6) over the preceding boxes.  flags may be
 * NULL (all fluid).  Levels must be defined in increasing order.
 * Replaces MakeNewLevelFromScratch's MultiFab definitions and
 * initialize_is_fluid (Source/LBM.cpp:1143-1262). */
mbg_status mbg_define_level(mbg_ctx* ctx, int lev, int nbox, const int* lohi,
                            const uint8_t* flags);

/* Number of valid cells of a level. */
mbg_status mbg_level_cells(const mbg_ctx* ctx, int lev, long long* ncells);

/* Upload / download f and g of a level (valid cells, FP64, 27 components).
 * Replaces Initializer::initialize (Source/IC.H:460-525) on the way in and
 * the MultiFab reads of plot/checkpoint output (Source/LBM.cpp:1629-1690)
 * on the way out.  f or g may be NULL to skip it. */
mbg_status mbg_set_state(mbg_ctx* ctx, int lev, const double* f, const double* g);
mbg_status mbg_get_state(mbg_ctx* ctx, int lev, double* f, double* g);

/* Macro fields of the current f, g (19 components in the order of
 * Source/Constants.H:8-31: rho, vel_x, vel_y, vel_z, vel_mag, two_rho_e,
 * QCorrX..Z, pxx, pyy, pzz, pxy, pxz, pyz, qx, qy, qz, temperature).
 * Replaces LBM::f_to_macrodata (Source/LBM.cpp:810-906). */
mbg_status mbg_get_macro(mbg_ctx* ctx, int lev, double* macro);

/* One coarse time step of the whole hierarchy: ghost fill of level 0, then
 * the recursive subcycled time_step (fine levels get 2 substeps per coarser
 * step, explosion before them, coalescence after them).  Replaces
 * LBM::evolve's loop body (Source/LBM.cpp:416-428) with time_step and
 * advance (Source/LBM.cpp:452-544) and FillPatchOps::fillpatch / physbc
 * (Source/FillPatchOps.H:75-159). */
mbg_status mbg_step(mbg_ctx* ctx, int nsteps);

/* One advance of a single level (stream + collide), without ghost fill
 * and without coalescence.  Replaces LBM::advance for a level without a
 * finer level (Source/LBM.cpp:523-544). */
mbg_status mbg_advance_level(mbg_ctx* ctx, int lev);

/* Fill the ghost cells of fine level lev > 0 from level lev-1 (explosion).
 * Replaces FillPatchOps::fillpatch for lev > 0 (Source/FillPatchOps.H:
 * 118-129, AMReX FillPatchTwoLevels with cell_cons_interp). */
mbg_status mbg_fillpatch(mbg_ctx* ctx, int lev);

/* Average fine level crse_lev+1 down onto level crse_lev over the covered
 * cells grown by crse_ng (0 or 1) (coalescence).  Replaces
 * LBM::average_down_to (Source/LBM.cpp:1571-1584) and
 * average_down_with_ghosts (Source/Utilities.cpp:5-28). */
mbg_status mbg_average_down(mbg_ctx* ctx, int crse_lev, int crse_ng);

/* Momentum-exchange force on embedded-boundary cells summed over all levels
 * (cells not covered by a finer level), FP64 accumulation in a fixed order
 * (per-block sums by warp shuffles, then one fixed-order sum of the blocks):
 * the same state gives the same bits on every call.  16-bit forms: the
 * stored populations (and fine levels' ghost fabs) decoded to FP64.
 * Replaces LBM::compute_eb_forces (Source/LBM.cpp:994-1044). */
mbg_status mbg_eb_forces(mbg_ctx* ctx, double out[3]);

/* Derived fields of the stored state of level lev (7 components in the
 * order of Source/Constants.H: vort_x, vort_y, vort_z, vort_mag, dQCorrX,
 * dQCorrY, dQCorrZ), layout of mbg_get_macro: the vorticity and the
 * q-correction gradients of the macro fields of the stored populations, by
 * the reference's central / one-sided differences with the physical 1/dx,
 * at fluid cells (0 elsewhere).  Replaces compute_derived and
 * compute_q_corrections (Source/LBM.cpp:909-991) after f_to_macrodata, as
 * the reference's output and restart paths call them. */
mbg_status mbg_get_derived(mbg_ctx* ctx, int lev, double* derived);

/* Conserved totals of the stored state over all levels, each cell counted on
 * the finest level that holds it and weighted by its volume, summed on the
 * device (FP64 form: FP64 throughout; 16-bit forms: each cell's 27 decoded
 * FP32 values in error-free FP32 TwoSum arithmetic, about 2^-48 relative,
 * then FP64 across cells): out = {mass, momentum x, y, z, sum of
 * 2 rho E}.  No counterpart in the reference (its only global reduction is
 * the EB-force sum, Source/LBM.cpp:1040); one reduction launch per level. */
mbg_status mbg_conserved(mbg_ctx* ctx, double out[5]);

/* State check (the debug scans of the plan's auxiliary subsystems; no
 * counterpart in the reference): every valid cell of every level is
 * scanned on the device.  A fluid cell must hold finite populations other
 * than the stream's -1 sentinel; a solid cell not overwritten by
 * coalescence the sentinel in every direction.  counts = {bad values at
 * fluid cells, bad values at solid cells}; first = {level, box, cell in the
 * box (x fastest), 2 q + lattice} of the first bad value in that order, or
 * -1 four times when there is none.  The 16-bit forms scan their decoded
 * state.  The state is not changed. */
mbg_status mbg_check_state(mbg_ctx* ctx, long long counts[2], long long first[4]);

/* Wait for all work queued on the context's stream; reports a latched
 * device-side error. */
mbg_status mbg_synchronize(mbg_ctx* ctx);

/* Number of kernel launches issued by the context since creation. */
long long mbg_launch_count(const mbg_ctx* ctx);

/* The CUDA stream every launch of the context goes to. */
void* mbg_stream(const mbg_ctx* ctx);

/* Per-kernel timing with CUDA events recorded around each launch on the
 * context's stream (off by default; enabling it resets the totals).
 * mbg_timing(k) reports kernel class k (0 .. mbg_timing_count()-1): its
 * name, the number of launches and their summed device time in ms. */
mbg_status mbg_set_timing(mbg_ctx* ctx, int enable);
int mbg_timing_count(void);
mbg_status mbg_timing(mbg_ctx* ctx, int k, const char** name, long long* launches, double* ms);

/* ---- autotuner ----------------------------------------------------------------
 * No counterpart in the reference.  The 16-bit forms have several
 * implementations of the level step: variant 0 runs it in two passes (Q_corr,
 * then collision) on two x-adjacent cells per thread with paired FP32
 * arithmetic wherever the box allows (even x extent, fluid one cell out), one
 * cell per thread elsewhere; variants 1-2 fuse it into one pass over runs of
 * 4 or 8 planes per thread block; variant 3 is the two-pass step on one cell
 * per thread with the collision pass limited to 80 registers (6 resident
 * blocks per SM).  mbg_autotune times every variant `reps` times on each
 * level's current data and keeps the fastest per level; the state is not
 * changed.  mbg_tuning reports a level's chosen variant and the mean time per
 * step of each variant in ms (0 where not timed).  mbg_set_variant makes a
 * level (lev >= 0) or every level (lev = -1) run the given variant.  FP64
 * contexts have one variant; the calls succeed, report variant 0 and accept
 * only variant 0. */
mbg_status mbg_autotune(mbg_ctx* ctx, int reps);
mbg_status mbg_tuning(mbg_ctx* ctx, int lev, int* variant, double ms[4]);
mbg_status mbg_set_variant(mbg_ctx* ctx, int lev, int variant);

/* ---- batched independent domains -----------------------------------------
 * No counterpart in the reference, which runs one domain per process.  Many
 * small periodic domains advance together, each with its own cell counts,
 * physical extent (the q-correction gradient uses its per-axis 1/dx),
 * viscosity and diffusivity; the gradient is one-sided at each domain's faces
 * as at the domain box of a single run.  Every launch covers all domains: a
 * pad fill and the step, the fused variants as a persistent grid walking a
 * device work list of column tiles (largest domains first).  Steps are
 * replayed from a CUDA graph of two steps captured on first use;
 * mbg_batch_autotune times the step variants on the live data (state
 * unchanged) and keeps the fastest.  16-bit forms only (common->precision
 * MBG_FP32C_F16S or MBG_FP32C_BF16S); the other common fields (dx_outer,
 * dt_outer, adiabatic_exponent, m_bar and the storage's reference state
 * rho_ref, t_ref, u_ref) apply to every domain.  Host state layout:
 * [domain][q][cell], cells x-fastest, domains in the order given; macro
 * fields [domain][19][cell] as mbg_get_macro.  A failed creation leaves its
 * message in mbg_last_error(NULL). */
typedef struct mbg_batch mbg_batch;
typedef struct mbg_domain {
    int n_cell[3];
    double prob_lo[3], prob_hi[3];
    double nu, alpha;
} mbg_domain;
mbg_status mbg_batch_create(const mbg_params* common, int ndom, const mbg_domain* doms, void* cuda_stream,
                            mbg_batch** out);
mbg_status mbg_batch_cells(const mbg_batch* b, long long* ncells);
mbg_status mbg_batch_set_state(mbg_batch* b, const double* f, const double* g);
mbg_status mbg_batch_get_state(mbg_batch* b, double* f, double* g);
mbg_status mbg_batch_get_macro(mbg_batch* b, double* out19);
mbg_status mbg_batch_step(mbg_batch* b, int nsteps);
mbg_status mbg_batch_autotune(mbg_batch* b, int reps);
mbg_status mbg_batch_tuning(mbg_batch* b, int* variant, double ms[4]);
mbg_status mbg_batch_synchronize(mbg_batch* b);
long long mbg_batch_launch_count(const mbg_batch* b);
void* mbg_batch_stream(const mbg_batch* b);
const char* mbg_batch_last_error(const mbg_batch* b);
void mbg_batch_destroy(mbg_batch* b);

/* ---- adjoint of the FP64 step ----------------------------------------------
 * No counterpart in the reference.  Gradient of a loss of the final
 * temperature field with respect to the initial temperature field, on one
 * fully periodic box (p->n_cell, prob_lo/hi, nu, alpha, dx_outer, dt_outer,
 * adiabatic_exponent, m_bar; precision MBG_FP64).  The initial state is the
 * equilibrium of (rho0, u0, T0(x)) as the reference's initializer builds it
 * (IC.H:474-519); a step is the reference's stream + collide.
 * mbg_adj_forward runs nsteps steps from T0 (host, one value per cell,
 * x fastest), checkpointing every K steps, and returns the final temperature
 * field (of the stored populations).  mbg_adj_backward takes dL/dT_final of
 * the last forward run and returns dL/dT0: the hand-written discrete adjoint
 * of every step, walked backwards segment by segment, each segment recomputed
 * from its checkpoint; FP64 throughout.  Memory: about (3 + nsteps/K + K)
 * states of 432 bytes per cell plus K x 136 bytes per cell. */
typedef struct mbg_adj mbg_adj;
mbg_status mbg_adj_create(const mbg_params* p, double rho0, const double u0[3], void* cuda_stream, mbg_adj** out);
mbg_status mbg_adj_forward(mbg_adj* a, const double* T0, int nsteps, int K, double* T_final);
mbg_status mbg_adj_backward(mbg_adj* a, const double* dL_dTfinal, double* dL_dT0);
long long mbg_adj_launch_count(const mbg_adj* a);
void* mbg_adj_stream(const mbg_adj* a);
const char* mbg_adj_last_error(const mbg_adj* a);
void mbg_adj_destroy(mbg_adj* a);

/* ---- step without device allocation --------------------------------------
 * No counterpart in the reference.  For callers that cannot let a library
 * allocate device memory: a host code that has given the GPU to its own
 * memory arena would risk an out-of-memory failure mid-run, and
 * cudaMalloc / cudaFree may synchronise the device, which a caller queueing
 * its time loop asynchronously on its own stream cannot accept.
 *
 * One FP64 step (stream, then collide and relax) of a single all-fluid box
 * that is periodic in every direction, of params->n_cell cells (at most
 * MBG_NOALLOC_MAX_CELLS in total), with no context and no allocation.
 * f_in, g_in, f_out, g_out are device arrays of 27 * ncells doubles in
 * [q][k][j][i] order; outputs must not alias inputs.  The scratch between
 * the two passes is a fixed array in the library's device image (4.5 MiB on
 * every GPU that loads the library, until exit), shared by all calls: calls
 * whose kernels overlap on the GPU race on it.  Each call looks up that
 * array's address on the current device (a host-side lookup, no device
 * work); the first call on a device may load the library's device code and
 * should come before any stream capture.  A box with any n_cell[d], or the
 * product, above the maximum is rejected with MBG_EINVAL.  Launches on
 * cuda_stream (NULL: the legacy default stream); errors are reported by
 * mbg_last_error(NULL). */
#define MBG_NOALLOC_MAX_CELLS 32768
mbg_status mbg_step_box_noalloc(const mbg_params* params, const double* f_in, const double* g_in,
                                double* f_out, double* g_out, void* cuda_stream);

/* ---- tagging and regrid ------------------------------------------------------
 * One refinement criterion of tagging.<name>.* (Source/LBM.cpp:302-396):
 * field 0..18 is a macro component in the order of mbg_get_macro, 19 is
 * is_fluid (component 0, which the reference's get_field copies for either
 * id field, Source/LBM.cpp:1536-1546); kind 0 tags every cell whose centre
 * lies in the box, 1 value_greater, 2 value_less (within the box if
 * has_box); the criterion applies while start_time <= time <= end_time and
 * the level is below max_level. */
#define MBG_MAX_TAGS 8
typedef struct mbg_tag {
    int field;
    int kind;
    double value;
    int has_box;
    double box_lo[3], box_hi[3];
    double start_time, end_time;
    int max_level;
} mbg_tag;

/* Tags (0/1 per valid cell, layout [box][k][j][i]) of level lev at simulated
 * time `time`, evaluated on the GPU from the level's macro data: in the FP64
 * form the moments its last collision started from (the reference's
 * m_macrodata), or those of the stored state when no step has run since the
 * state was set; in the 16-bit forms the moments of the stored state.
 * Replaces LBM::ErrorEst (Source/LBM.cpp:1597-1611) with AMReX's
 * AMRErrorTag. */
mbg_status mbg_tag_cells(mbg_ctx* ctx, int lev, const mbg_tag* tags, int ntags, double time, uint8_t* out);

/* Replace levels first_lev .. of the hierarchy by nlev levels with new box
 * arrays (nbox[m] boxes each, lohi concatenated over the levels, flags in the
 * layout of mbg_define_level concatenated likewise); levels beyond them are
 * dropped and their device memory freed.  Each new level's cells keep the
 * old level's values where an old box held them and are interpolated from
 * the coarser level (conservative linear, on the GPU) elsewhere; solid cells
 * start at 0.  Replaces LBM::RemakeLevel / MakeNewLevelFromCoarse /
 * ClearLevel (Source/LBM.cpp:1088-1140, 1302-1379). */
mbg_status mbg_regrid(mbg_ctx* ctx, int first_lev, int nlev, const int* nbox, const int* lohi,
                      const uint8_t* flags);

/* ---- embedded-boundary geometry -------------------------------------------
 * eb2.geom_type and its keys (Source/EB.cpp:5-38, Source/Geometry.cpp:5-200):
 * the AMReX built-in sphere, box, cylinder and plane and the reference's own
 * rotated box, rotated cylinder and extruded triangles. */
enum {
    MBG_GEOM_ALL_REGULAR = 0, MBG_GEOM_SPHERE = 1, MBG_GEOM_BOX = 2, MBG_GEOM_CYLINDER = 3,
    MBG_GEOM_PLANE = 4, MBG_GEOM_ROTATED_BOX = 5, MBG_GEOM_ROTATED_CYLINDER = 6,
    MBG_GEOM_EXTRUDED_TRIANGLES = 7
};
typedef struct mbg_geometry {
    int type;                   /* MBG_GEOM_*                                       */
    int has_fluid_inside;       /* eb2.{sphere,box,cylinder}_has_fluid_inside       */
    double center[3];           /* eb2.sphere_center / eb2.cylinder_center          */
    double radius;              /* eb2.sphere_radius / eb2.cylinder_radius          */
    double height;              /* eb2.cylinder_height (<= 0: unbounded)            */
    int direction;              /* eb2.cylinder_direction                           */
    double lo[3], hi[3];        /* eb2.box_lo, eb2.box_hi                           */
    double point[3], normal[3]; /* eb2.plane_point, eb2.plane_normal                */
    double rotation_deg;        /* eb2.box_rotation / eb2.cylinder_rotation         */
    int rotation_axis;          /* eb2.box_rotation_axe / eb2.cylinder_rotation_axe */
    double rotation_center[3];  /* eb2.box_rotation_center                          */
    int ntri;                   /* extruded_triangles.num_tri (at most 5)           */
    double tri[5][3][2];        /* extruded_triangles.tri_<t>_point_<p> (x, y)      */
} mbg_geometry;

/* is_fluid flags (bit 0 is_fluid, bit 1 eb_boundary) of level lev's boxes,
 * each grown by 3, in the layout mbg_define_level takes, evaluated on the
 * GPU on cuda_stream: a cell is covered when the geometry's implicit
 * function puts all 8 of its corners in the body.  Uses params' n_cell,
 * prob_lo/hi and is_periodic.  Replaces the EB2 build and
 * initialize_is_fluid (Source/EB.cpp:5-38, Source/LBM.cpp:1213-1262).
 * Errors are reported by mbg_last_error(NULL). */
mbg_status mbg_geometry_flags(const mbg_geometry* geom, const mbg_params* params, int lev, int nbox,
                              const int* lohi, uint8_t* flags, void* cuda_stream);

/* ---- AMReX-format files (host only, no device work) ------------------------
 * Errors are reported by mbg_last_error(NULL).
 *
 * mbg_write_plotfile writes an AMReX plotfile directory (HyperCLaw-V1.1
 * Header, Level_<l>/Cell_H and Cell_D_00000) of nlev levels at ratio 2:
 * nbox[l] boxes per level, lohi the boxes of all levels concatenated (6 ints
 * each, inclusive, in the level's index space), n_cell the level-0 domain,
 * ncomp components named varnames, data[l] the level's values [box][comp]
 * [k][j][i].  Replaces amrex::WriteMultiLevelPlotfile as LBM::write_plot_file
 * calls it (Source/LBM.cpp:1677-1690). */
mbg_status mbg_write_plotfile(const char* dir, int nlev, const int* nbox, const int* lohi, const int* n_cell,
                              const double* prob_lo, const double* prob_hi, int ncomp,
                              const char* const* varnames, const double* const* data, double time,
                              const int* level_steps);

/* A VisMF multifab <prefix>_H + <prefix>_D_00000 of nbox boxes (valid cells,
 * no ghost cells), data [box][comp][k][j][i].  mbg_read_multifab reads one
 * back into the same layout; the file's boxes must equal lohi (files with
 * ghost cells are accepted, their valid region is kept).  Replace
 * amrex::VisMF::Write / VisMF::Read of the checkpoint's f and g
 * (Source/LBM.cpp:1770-1782, 1883-1893). */
mbg_status mbg_write_multifab(const char* prefix, int nbox, const int* lohi, int ncomp, const double* data);
mbg_status mbg_read_multifab(const char* prefix, int nbox, const int* lohi, int ncomp, double* data);

/* ---- host drop-in driver ----------------------------------------------
 * The reference's LBM/AmrCore driver (Source/LBM.H:25-319, main.cpp:10-25)
 * on top of the entry points above: reads an inputs file with the
 * reference's keys (amr.*, geometry.*, lbm.*, ic_<type>.*,
 * velocity_bc_<type>.*, eb2.*, tagging.*) plus "key=value" overrides, builds
 * static grids, EB flags and the initial state, and runs the time loop. */
typedef struct mbg_lbm mbg_lbm;

/* Parse inputs text (and overrides) and select the IC / velocity-BC
 * functors.  Replaces LBM::LBM() and read_parameters (Source/LBM.cpp:6-300)
 * with set_ics / set_bcs (LBM.cpp:1382-1476). */
mbg_status mbg_lbm_create(const char* inputs_text, int n_overrides, const char* const* overrides, mbg_lbm** out);

/* Grids, flags, initial state and the initial average_down.  Replaces
 * LBM::init_data (Source/LBM.cpp:155-194). */
mbg_status mbg_lbm_init(mbg_lbm* h);

/* nsteps coarse steps (nsteps <= 0: until max_step / stop_time), with
 * forces and plotfiles at their intervals.  Replaces LBM::evolve
 * (Source/LBM.cpp:398-448). */
mbg_status mbg_lbm_evolve(mbg_lbm* h, int nsteps);

/* Host-only part of init_data: grids (level 0 chopped by
 * amr.max_grid_size, finer levels from tagging.*) and is_fluid flags.
 * Replaces AmrCore::InitFromScratch's grid creation with
 * initialize_is_fluid (Source/LBM.cpp:165, 1213-1262). */
mbg_status mbg_lbm_prepare(mbg_lbm* h);

/* Initial f and g of level lev on the host (valid cells; layout of
 * mbg_set_state), from the selected IC functor and fill_f_inside_eb.
 * Replaces Initializer::initialize (Source/IC.H:460-525) and
 * LBM::fill_f_inside_eb (Source/LBM.cpp:1278-1298). */
mbg_status mbg_lbm_initial_state(mbg_lbm* h, int lev, double* f, double* g);

/* The level-step context the driver runs on (owned by the driver). */
mbg_ctx* mbg_lbm_context(mbg_lbm* h);

/* Grids and is_fluid flags the driver built (layout of mbg_define_level). */
int mbg_lbm_num_levels(const mbg_lbm* h);
mbg_status mbg_lbm_level_boxes(const mbg_lbm* h, int lev, int* lohi, int cap, int* nbox);
mbg_status mbg_lbm_level_flags(const mbg_lbm* h, int lev, uint8_t* out, long long cap, long long* n);

/* AMReX plotfile of the current state: the 19 macro fields of the stored
 * populations, f and g (lbm.save_streaming), the 7 derived fields of
 * mbg_get_derived (lbm.save_derived) and is_fluid / eb_boundary, with the
 * reference's variable names.  Replaces LBM::write_plot_file
 * (Source/LBM.cpp:1613-1690). */
mbg_status mbg_lbm_write_plotfile(mbg_lbm* h, const char* name);

/* Checkpoint directory of the current state: Header (title, finest level,
 * steps, dts and times per level, box arrays) and Level_<l>/f_00, g_00
 * multifabs.  A run whose inputs set amr.restart = <dir> resumes from it in
 * mbg_lbm_init (the grids must be those the inputs build).  Replaces
 * LBM::write_checkpoint_file / read_checkpoint_file
 * (Source/LBM.cpp:1692-1916). */
mbg_status mbg_lbm_write_checkpoint(mbg_lbm* h, const char* name);

/* Regrid now: tag every level below amr.max_level on the GPU with the
 * tagging.* criteria (mbg_tag_cells), rebuild the fine grids from the tags
 * (buffered by amr.n_error_buf, clustered on amr.blocking_factor blocks,
 * chopped by amr.max_grid_size, nested), and remake the levels whose grids
 * changed (mbg_regrid).  mbg_lbm_evolve does this before every coarse step
 * whose count is a positive multiple of amr.regrid_int, as time_step(0)
 * does (Source/LBM.cpp:456-479); finer levels' own regrid points inside a
 * coarse step are not taken. */
mbg_status mbg_lbm_regrid(mbg_lbm* h);

/* Coarse steps taken and the simulated time of the driver. */
mbg_status mbg_lbm_step_time(const mbg_lbm* h, int* step, double* time);

const char* mbg_lbm_last_error(const mbg_lbm* h);
void mbg_lbm_destroy(mbg_lbm* h);

#ifdef __cplusplus
}
#endif
#endif /* MARBLES_GB300_H */
