/*
 * fsi_gb300.h -- C ABI of the GB300 (sm_103a) coupled LBM-MPM timestep.
 *
 * Each entry point replaces one or more Taichi kernels of the reference
 * lizhuoh9/taichi-mpm-lbm (cited as file:line). Conventions:
 *   - all array arguments are device pointers owned by the caller (the Python
 *     package allocates them as torch CUDA tensors); the library allocates
 *     device memory only for the scratch of a context or batch, in their
 *     create / set-up calls, and frees it in their destroy calls;
 *   - descriptor structs and small `const float*` parameter vectors marked
 *     "host" are read on the host during the call;
 *   - work is enqueued on `stream` (a cudaStream_t passed as void*, NULL = the
 *     legacy default stream) and runs asynchronously;
 *   - the return value is an FSI_* status; on failure fsi_last_error()
 *     returns a message. No C++ exception crosses this boundary.
 *
 * Data layouts (N = nx*ny*nz cells, linear cell c = (i*ny + j)*nz + k, i.e.
 * the C order of the reference's numpy arrays):
 *   pops    float[19][N]  populations, structure of arrays, AA-pattern storage
 *   macro   float[N][4]   (ux, uy, uz, rho) per cell
 *   force   float[3][N]   body force density, structure of arrays
 *   flags   uint32[N]     bit 0 solid; bit q (1..18) neighbour x+e_q solid;
 *                         bit 20/21 x=0 / x=nx-1 face cell; bit 22+4a+2b+c corner
 *                         neighbour x+(2a-1,2b-1,2c-1) solid (neighbours wrap
 *                         periodically); built by fsi_lbm_build_flags, which the
 *                         coupling entry points rely on
 *   solid   int32[N]      0/1 solid mask as the reference stores it
 */
#ifndef FSI_GB300_H
#define FSI_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FSI_OK 0
#define FSI_ERR_INVALID_ARG 1
#define FSI_ERR_CUDA 2
#define FSI_ERR_GUARD 3
#define FSI_ERR_TIMEOUT 4
#define FSI_ERR_UNSUPPORTED 5

#define FSI_ABI_VERSION 5

/* Library ABI version (FSI_ABI_VERSION). No reference counterpart. */
int fsi_abi_version(void);

/* Copies the last error message of the calling thread into buf (NUL-terminated);
 * returns the message length. No reference counterpart (Taichi raises Python
 * exceptions directly). */
size_t fsi_last_error(char* buf, size_t len);

/* ------------------------------------------------------------------ LBM -- */

/* Lattice description. Replaces the scalar fields of LBMSolver3D
 * (fsi/lbm3d.py:110-191): relaxation rates, rho0 and the x-face conditions. */
typedef struct fsi_lbm_desc {
  int32_t nx, ny, nz;
  int32_t bc_mode_left;   /* x = 0 face: 0 periodic, 1 pressure, 2 velocity (lbm3d.py:16-27);
                             3 velocity with every population read from before the update
                             (no reference counterpart; the reference updates in place) */
  int32_t bc_mode_right;  /* x = nx-1 face, same codes */
  float s[19];            /* MRT relaxation rates S_k (lbm3d.py:141-168) */
  float rho0;
  float bc_rho_left, bc_rho_right;
  float bc_vel_left[3], bc_vel_right[3];
  int32_t storage;     /* FSI_STORAGE_*: element type of the population array */
  int32_t arithmetic;  /* FSI_ARITH_*: operation order of the collision */
} fsi_lbm_desc;

/* Population storage. F32 holds f_q; F16 holds (f_q - w_q rho0) * 4096 as IEEE half;
 * BF16 holds f_q - w_q rho0 as bfloat16. The population array has 19 * N elements of
 * that type in every form; all arithmetic is float32. No reference counterpart: the
 * reference stores float32 (lbm3d.py:117-122). */
#define FSI_STORAGE_F32 0
#define FSI_STORAGE_F16 1
#define FSI_STORAGE_BF16 2
/* Collision arithmetic. EXACT reproduces the reference's float32 operations in its
 * order (bit-identical populations); FAST evaluates the same operator with fused
 * multiply-adds and parity-split moments (about 2.5x fewer operations, results within
 * float32 rounding). F16/BF16 storage requires FAST. */
#define FSI_ARITH_EXACT 0
#define FSI_ARITH_FAST 1

/* Builds the per-cell flag word from the normalised 0/1 mask.
 * Replaces the neighbour tests of LBMSolver3D.stream (fsi/lbm3d.py:335-361),
 * evaluated once at initialisation instead of every step. */
int fsi_lbm_build_flags(const fsi_lbm_desc* desc, const int32_t* solid, uint32_t* flags,
                        void* stream);

/* Equilibrium initialisation: rho = rho0, u = u0 (0 on solid cells),
 * populations = feq(rho0, u). u0 is host float[3].
 * Replaces LBMSolver3D.init_fields (fsi/lbm3d.py:256-267). */
int fsi_lbm_init_fields(const fsi_lbm_desc* desc, const uint32_t* flags, const float* u0,
                        void* pops, float* macro, void* stream);

/* One lattice step: collide (MRT + Guo forcing) and stream (half-way
 * bounce-back, periodic wrap) in one in-place AA-pattern pass, followed by the
 * x-face conditions. `steps_done` is the number of steps already taken (its
 * parity selects the AA access pattern).
 *   force_prev == NULL: rho and u of the current state are read from `macro`
 *                       (valid after fsi_lbm_init_fields / fsi_lbm_update_macro);
 *   force_prev != NULL: they are recomputed in-register from the populations and
 *                       force_prev, the force the previous step used, exactly as
 *                       update_macro would have stored them.
 * `macro` is left stale except on x-face cells; call fsi_lbm_update_macro to
 * materialise rho and u of the new state.
 * Replaces LBMSolver3D.collide/stream/apply_boundary (fsi/lbm3d.py:314-407,
 * called from step() at lbm3d.py:427-433). */
int fsi_lbm_step(const fsi_lbm_desc* desc, void* pops, float* macro, const float* force,
                 const float* force_prev, const uint32_t* flags, int64_t steps_done,
                 void* stream);

/* rho = sum f, u = sum e f / rho + force / (2 rho) on fluid cells; rho0 and 0
 * on solid cells. `force` is the force of the last step.
 * Replaces LBMSolver3D.update_macro (fsi/lbm3d.py:409-425). */
int fsi_lbm_update_macro(const fsi_lbm_desc* desc, const void* pops, const float* force,
                         const uint32_t* flags, int64_t steps_done, float* macro,
                         void* stream);

/* Writes the post-stream distribution in the reference layout float[N][19].
 * Replaces LBMSolver3D.distribution_numpy (fsi/lbm3d.py:444-445). */
int fsi_lbm_distribution(const fsi_lbm_desc* desc, const void* pops, const uint32_t* flags,
                         int64_t steps_done, float* out, void* stream);

/* Force-field operations on float[3][N] (value is host float[3]):
 *   FSI_FORCE_CLEAR     out = 0                         (lbm3d.py:499-502)
 *   FSI_FORCE_SET       out = fluid ? value : 0          (lbm3d.py:504-519)
 *   FSI_FORCE_ADD       out = fluid ? in + value : 0     (lbm3d.py:521-528)
 *   FSI_FORCE_ZERO_SOLID out = fluid ? in : 0            (lbm3d.py:530-534)
 * `in` may equal `out`. */
#define FSI_FORCE_CLEAR 0
#define FSI_FORCE_SET 1
#define FSI_FORCE_ADD 2
#define FSI_FORCE_ZERO_SOLID 3
int fsi_lbm_force_op(const fsi_lbm_desc* desc, const uint32_t* flags, int op, const float* in,
                     const float* value, float* out, void* stream);

/* Lattice diagnostics into device double[8]:
 *   [0] sum of rho over fluid cells            (total_mass, lbm3d.py:450-453)
 *   [1] max |u| over all cells                 (max_velocity_norm, lbm3d.py:455-457)
 *   [2..4] sum of force over fluid cells       (total_force, lbm3d.py:480-483)
 * `out` must be zero-initialised except that it is overwritten here. */
int fsi_lbm_reduce(const fsi_lbm_desc* desc, const float* macro, const float* force,
                   const uint32_t* flags, double* out, void* stream);

/* fsi_lbm_update_macro fused with the two per-step runner diagnostics: writes `macro` and
 * device double out[0] = sum of rho over fluid cells, out[1] = max |u| over all cells
 * (LBMSolver3D.total_mass / max_velocity_norm, lbm3d.py:450-457, as called by
 * FSISimulation.diagnostics, simulation.py:117-147), in one pass over the populations. */
int fsi_lbm_macro_diagnostics(const fsi_lbm_desc* desc, const void* pops, const float* force,
                              const uint32_t* flags, int64_t steps_done, float* macro,
                              double* out, void* stream);

/* ------------------------------------------------------------------ MPM -- */

/* Solid (MLS-MPM) description. Replaces the scalar fields of MPMSolver3D
 * (fsi/mpm3d.py:17-67). mu and lam are the Lame parameters of mpm3d.py:33-38;
 * clamp_lower / clamp_upper the position limits of mpm3d.py:320-328. */
typedef struct fsi_mpm_desc {
  int32_t nx, ny, nz;
  int32_t num_particles; /* particles live in slots [0, num_particles) */
  float dt, dx, inv_dx;
  float mu, lam;
  float gravity[3];
  float boundary_damping;
  int32_t boundary_width;
  int32_t apic;
  float clamp_lower;
  float clamp_upper[3];
  int32_t material; /* FSI_MATERIAL_*; the reference's model is fixed-corotated */
  /* Launch tuning of the tiled scatter (no reference counterpart; fsi.autotune sets them):
   * threads per block of P2G and G2P, 128, 256 or 512 (0: 256), which sets the particles whose
   * stencils share one shared-memory tile; and where a coupled tiled substep forms the
   * coupling force: 0 by particle count, 1 inside P2G, 2 in a kernel of its own first, 3 in
   * a force kernel and a spread kernel of their own first. */
  int32_t launch_threads;
  int32_t coupling_fold;
} fsi_mpm_desc;

/* Constitutive models. FIXED_COROTATED is the reference's
 * 2 mu (F - R) F^T + lam J (J - 1) I (mpm3d.py:247-251); NEO_HOOKEAN is the
 * compressible mu (F F^T - I) + lam ln(J) I, an extension with no reference
 * counterpart (its oracle is the CPU restatement). */
#define FSI_MATERIAL_FIXED_COROTATED 0
#define FSI_MATERIAL_NEO_HOOKEAN 1

/* Particle arrays, structure of arrays with component stride `capacity`:
 * x, v, force float[3][capacity]; C, F float[9][capacity] (row-major 3x3
 * components); mass, volume float[capacity]; active int32[capacity].
 * Replaces the particle fields of mpm3d.py:44-55. */
typedef struct fsi_particles {
  float* x;
  float* v;
  float* C;
  float* F;
  float* mass;
  float* volume;
  int32_t* active;
  float* force;
  int64_t capacity;
  float* mu;  /* per-particle Lame parameters float[capacity], or both NULL to use the */
  float* lam; /* descriptor's scalars (the reference has one material per solver) */
} fsi_particles;

/* One MPM substep: P2G (deformation update, fixed-corotated stress, 27-node
 * scatter), grid update and G2P (APIC gather, advection, clamp).
 * `grid` is float[N][4] (momentum xyz, mass), 16-byte aligned, all zero on
 * entry and left all zero on return; `dirty` is uint8[ceil(nx/4)*ceil(ny/4)*
 * ceil(nz/4)], zero on entry and on return. dt is desc->dt.
 * Replaces MPMSolver3D.clear_grid/p2g/grid_op/g2p (fsi/mpm3d.py:189-318). */
int fsi_mpm_substep(const fsi_mpm_desc* desc, const fsi_particles* particles, float* grid,
                    uint8_t* dirty, void* stream);

/* fsi_mpm_substep for callers that cannot allocate device memory (no counterpart in the
 * reference, which allocates its grid as Taichi fields). Hosts such as real-time loops that
 * may not take the device synchronisation of cudaMalloc, plugins inside an application that
 * owns the device memory pool, or plain FFI callers without a device allocator pass only the
 * particles; the grid and dirty-block map live in one static device array of this library
 * (FSI_NOALLOC_MAX_NODES float4 nodes + FSI_NOALLOC_MAX_BLOCKS bytes, about 4 MB held on every
 * GPU that loads the library until exit). Grids above either limit are rejected with
 * FSI_ERR_INVALID_ARG. The first call in a CUDA context (per device and per context, e.g.
 * again after cudaDeviceReset) looks up the array's device address with cudaGetSymbolAddress
 * and caches it under the context's ID; make that first call before any stream capture. All calls share the array: each call clears the part it uses, and calls
 * whose work overlaps on the GPU (other streams, other threads) race on it. Nothing is
 * allocated or freed. */
#define FSI_NOALLOC_MAX_NODES (64 * 64 * 64)
#define FSI_NOALLOC_MAX_BLOCKS 32768
int fsi_mpm_substep_noalloc(const fsi_mpm_desc* desc, const fsi_particles* particles, void* stream);

/* Bytes of the workspace that fsi_mpm_substep_sorted and fsi_coupled_substep need for this
 * grid and a particle capacity: the per-cell and per-tile counts and starts of the particle
 * sort, the sorted order and a 128-byte record per particle. The workspace is one device
 * buffer, 256-byte aligned and zero-filled once before its first use; the substeps leave its
 * count arrays zero again. No reference counterpart (the reference does not sort). */
int fsi_mpm_workspace_bytes(const fsi_mpm_desc* desc, int64_t capacity, int64_t* bytes);

/* One MPM substep with a deterministic scatter: the particles are sorted by base cell
 * trunc(x / dx - 0.5) every substep, each cell's 27 stencil partials are summed over its
 * particles in ascending index, and each node adds its cells' partials in ascending cell
 * index; node tiles are owned by one thread block each, so the grid is written with plain
 * stores and no atomics, and results repeat bit for bit from run to run. `grid` is float[N][4]
 * (16-byte aligned); it need not be zero on entry and holds the substep's momentum and mass
 * on the touched nodes on return (other nodes keep stale values). Same physics as
 * fsi_mpm_substep; replaces MPMSolver3D.clear_grid/p2g/grid_op/g2p (fsi/mpm3d.py:189-318). */
int fsi_mpm_substep_sorted(const fsi_mpm_desc* desc, const fsi_particles* particles, float* grid,
                           void* workspace, int64_t workspace_bytes, void* stream);

/* Rotation R of the polar decomposition of n row-major 3x3 matrices (float[n][9]).
 * Replaces the ti.svd call of MPMSolver3D.p2g (fsi/mpm3d.py:245-246). */
int fsi_mpm_polar(const float* F, float* R, int64_t n, void* stream);

/* Particle-to-cell indices base = trunc(x * inv_dx - 0.5) as int32[n][3].
 * Exposes the index computation of mpm3d.py:239 and coupling.py:343-344. */
int fsi_mpm_base_cells(const fsi_mpm_desc* desc, const fsi_particles* particles, int32_t* out,
                       void* stream);

/* Particle diagnostics into device double[8]: [0] sum m, [1..3] sum m x,
 * [4] max |v|, [5..7] sum particle force. Replaces the host reductions of
 * center_of_mass / max_velocity_norm (mpm3d.py:353-368) and
 * total_particle_coupling_force (coupling.py:226-227). `reserved` must be NULL. */
int fsi_mpm_reduce(const fsi_mpm_desc* desc, const fsi_particles* particles, double* out,
                   void* reserved, void* stream);

/* ------------------------------------------------------------- coupling -- */

/* Coupling parameters (CouplingConfig, fsi/config.py:141-196, as the fields of
 * LBMMpmCoupler, fsi/coupling.py:58-133). gamma_eff is the ramped gamma of
 * coupling.py:321-330 for the current coupled step. */
typedef struct fsi_coupling_desc {
  float gamma_eff;
  float dt_ratio;
  float cell_volume;
  float inv_dx;
  float min_valid_weight;
  float rel_limit;
  float force_limit;
  int32_t build_fraction;
  int32_t use_rel_limit;
  int32_t use_force_limit;
  int32_t ib_enabled;
  float ib_drag;
  float ib_threshold;
  int32_t ib_use_max;
  float ib_max_force;
  int32_t contact_enabled;
  float contact_threshold;
  float contact_damping;
} fsi_coupling_desc;

/* Device-side counters of one coupled step (coupling.py:79-92). */
typedef struct fsi_coupling_counters {
  int32_t unsupported, partial, clipped;
  int32_t contact_candidates, contact_damped;
  int32_t ib_active, ib_clipped;
  int32_t reserved;
  float ib_total[4];
} fsi_coupling_counters;

/* Penalty coupling of every particle against the current fluid velocity
 * (`macro`, float[N][4]): writes particle force, valid weight and coupling
 * mask (0 for inactive particles), increments the unsupported / partial /
 * clipped counters, and adds the fluid reaction (xyz) and, if
 * desc->build_fraction, the solid volume fraction (w) into `accum` float[N][4].
 * Replaces _compute_coupling_forces_kernel (fsi/coupling.py:332-406). */
int fsi_coupling_forces(const fsi_coupling_desc* desc, const fsi_mpm_desc* mpm,
                        const fsi_particles* particles, const float* macro,
                        const uint32_t* flags, float* accum, float* valid_weight,
                        int32_t* coupling_mask, void* counters, void* stream);

/* One coupled MPM substep: fsi_coupling_forces followed by fsi_mpm_substep_sorted, with the
 * fluid reaction and solid-fraction spread folded into the sorted scatter (same order rule:
 * per-cell partials over the cell's coupled particles, then ascending cell index per fluid
 * node, added to `accum`'s current values) and the per-particle coupling force computed in
 * the same pass as the stress. Zeroes and then fills the unsupported / partial / clipped
 * counters. Replaces one iteration of the substep loop of LBMMpmCoupler.step
 * (fsi/coupling.py:146-158): _compute_coupling_forces_kernel and MPMSolver3D.substep. */
int fsi_coupled_substep(const fsi_coupling_desc* coupling, const fsi_mpm_desc* desc,
                        const fsi_particles* particles, const float* macro, const uint32_t* flags,
                        float* accum, float* valid_weight, int32_t* coupling_mask, void* counters,
                        float* grid, void* workspace, int64_t workspace_bytes, void* stream);

/* One coupled MPM substep on the tiled scatter of fsi_mpm_substep: fsi_coupling_forces and
 * P2G, then grid update + G2P and the block clear. Under 2 x 152 x 256 particles the coupling
 * is folded into P2G (each particle's coupling force formed first, then the stress and the
 * 27-node scatter, the fluid reaction and solid fraction reduced into `accum` beside it);
 * above it the coupling runs as its own lighter kernel before P2G. Zeroes and then fills the unsupported /
 * partial / clipped counters. `grid` and `dirty` as for fsi_mpm_substep. Replaces one
 * iteration of the substep loop of LBMMpmCoupler.step (fsi/coupling.py:146-158):
 * _compute_coupling_forces_kernel and MPMSolver3D.substep. */
int fsi_coupled_substep_tiled(const fsi_coupling_desc* coupling, const fsi_mpm_desc* desc,
                              const fsi_particles* particles, const float* macro,
                              const uint32_t* flags, float* accum, float* valid_weight,
                              int32_t* coupling_mask, void* counters, float* grid,
                              uint8_t* dirty, void* stream);

/* Rebuilds the LBM force field float[3][N] for the next lattice step:
 *   FSI_ASSEMBLE_CLAMP_FRACTION  accum.w = min(accum.w, 1)   (coupling.py:408-411)
 *   (always)                     force = fluid ? base : 0     (lbm3d.py:504-510)
 *   FSI_ASSEMBLE_COUPLING        force += accum.xyz on fluid  (coupling.py:413-419)
 *   FSI_ASSEMBLE_IB              Brinkman drag into ib_force float[3][N], counters
 *                                and totals, force += ib      (coupling.py:421-461)
 * base_force is host float[3], or with FSI_ASSEMBLE_BASE_ON_DEVICE a device float[3] that
 * the kernel reads (a force that changes between replays of a captured CUDA graph); force may
 * be NULL to update accum/ib_force only. IB counters/totals must be zeroed by the caller. */
#define FSI_ASSEMBLE_CLAMP_FRACTION 1
#define FSI_ASSEMBLE_COUPLING 2
#define FSI_ASSEMBLE_IB 4
#define FSI_ASSEMBLE_BASE_ON_DEVICE 8
int fsi_coupling_assemble(const fsi_coupling_desc* desc, const fsi_lbm_desc* lbm,
                          const uint32_t* flags, const float* base_force, int mode, float* accum,
                          const float* macro, float* force, float* ib_force, void* counters,
                          void* stream);

/* fsi_coupling_assemble that also sets device double reaction[3] (zeroed here) to the sum
 * of the fluid reaction accum.xyz over fluid cells, read in the same pass over the
 * accumulator: the value fsi_coupling_reduce gives for the accumulator that the assembly
 * read. Fuses total_fluid_coupling_force (coupling.py:229-232) into the assembly of
 * coupling.py:408-461 for runners that report it every step (simulation.py:117-147). */
int fsi_coupling_assemble_sum(const fsi_coupling_desc* desc, const fsi_lbm_desc* lbm,
                              const uint32_t* flags, const float* base_force, int mode,
                              float* accum, const float* macro, float* force, float* ib_force,
                              void* counters, double* reaction, void* stream);

/* Contact detection and damping after an MPM substep; resets and fills the
 * contact counters and the contact mask.
 * Replaces _compute_contact_diagnostics_kernel (fsi/coupling.py:463-496). */
int fsi_contact(const fsi_coupling_desc* desc, const fsi_mpm_desc* mpm,
                const fsi_particles* particles, const float* accum, const uint32_t* flags,
                int32_t* contact_mask, void* counters, void* stream);

/* Sum of the fluid reaction force density over fluid cells into device
 * double[4] ([0..2]). Replaces total_fluid_coupling_force (coupling.py:229-232). */
int fsi_coupling_reduce(const fsi_lbm_desc* lbm, const float* accum, const uint32_t* flags,
                        double* out, void* stream);

/* The coupled runner's per-step diagnostics in one launch, into device double out[22]
 * (zeroed here): [0] sum of particle mass, [1..3] sum of m x, [4] max |v|, [5..7] sum of the
 * particle coupling force (as fsi_mpm_reduce); [8..10] sum of the fluid reaction over fluid
 * cells (as fsi_coupling_reduce; 0 when accum is NULL); [11..18] the eight int32 counters of
 * fsi_coupling_counters and [19..21] its IB force totals (0 when counters is NULL). Replaces
 * the host reductions behind FSISimulation.diagnostics (simulation.py:117-147), which the
 * caller reads back with one copy. */
int fsi_coupled_diagnostics(const fsi_mpm_desc* mpm, const fsi_particles* particles,
                            const fsi_lbm_desc* lbm, const float* accum, const uint32_t* flags,
                            const void* counters, double* out, void* stream);

/* ------------------------------------------------------------- one coupled scene
 * The coupled timestep in one call, for hosts that do not run the Python package (C, C++,
 * FFI). A context binds the caller's device buffers of one scene and owns only scratch (the
 * MPM grid and block map or the sorted-scatter workspace); fsi_coupled_step then performs
 * LBMMpmCoupler.step (fsi/coupling.py:135-173) with the lattice bookkeeping of
 * LBMSolver3D.step (fsi/lbm3d.py:427-433): the same launches, in the same order and with the
 * same arguments as the Python package, so both give the same results. */
typedef struct fsi_ctx fsi_ctx;

/* Scatter order of the MPM substep (MPMConfig.p2g_mode). */
#define FSI_P2G_ATOMIC 0 /* fsi_mpm_substep / fsi_coupled_substep_tiled */
#define FSI_P2G_SORTED 1 /* fsi_mpm_substep_sorted / fsi_coupled_substep */

typedef struct fsi_scene_desc {
  fsi_lbm_desc lbm;
  fsi_mpm_desc mpm;           /* dt is set per substep to float32(lbm_dt / substeps) */
  fsi_coupling_desc coupling; /* gamma_eff, dt_ratio, build_fraction: set per step / substep */
  float base_force[3];        /* LBMConfig.force, the lattice's uniform body force */
  float gamma;                /* CouplingConfig.gamma, ramped over gamma_ramp_steps */
  int32_t gamma_ramp_steps;
  int32_t coupling_enabled;          /* CouplingConfig.enabled */
  int32_t build_solid_fraction;      /* CouplingConfig.build_solid_volume_fraction */
  int32_t contact_enabled;           /* CouplingConfig.contact_enabled */
  int32_t immersed_boundary_enabled; /* CouplingConfig.immersed_boundary_enabled */
  int32_t p2g_mode;                  /* FSI_P2G_* */
} fsi_scene_desc;

/* Device buffers of the scene, owned by the caller; they must outlive the context. */
typedef struct fsi_scene_buffers {
  void* pops;           /* populations [19][N] in lbm.storage (fsi_lbm_init_fields) */
  float* macro;         /* float[N][4] */
  float* force[2];      /* two float[3][N] force buffers; force[0] holds the current force */
  uint32_t* flags;      /* fsi_lbm_build_flags */
  fsi_particles particles;
  float* accum;         /* float[N][4]: the coupling fields of the last step */
  float* ib_force;      /* float[3][N], or NULL without the immersed boundary */
  float* valid_weight;  /* float[capacity] */
  int32_t* coupling_mask; /* int32[capacity] */
  int32_t* contact_mask;  /* int32[capacity], or NULL without contact */
  void* counters;       /* fsi_coupling_counters */
} fsi_scene_buffers;

/* Validates the description and buffers and allocates the context's scratch (device memory,
 * zero-filled; synchronous: call outside stream capture). The lattice starts as
 * fsi_lbm_init_fields leaves it: no step taken, macro current, force[0] current; the
 * coupled-step counter (the gamma ramp's) starts at 0. */
int fsi_ctx_create(const fsi_scene_desc* desc, const fsi_scene_buffers* buffers, fsi_ctx** ctx);
int fsi_ctx_destroy(fsi_ctx* ctx);

/* Host bookkeeping of the context: lattice steps taken (their parity selects the AA access
 * pattern), whether `macro` is current, the force buffers of the next and of the last
 * lattice step (-1: none), and coupled steps taken. set_state adopts the state of a lattice
 * stepped elsewhere (e.g. by the Python package on the same buffers). */
int fsi_ctx_get_state(const fsi_ctx* ctx, int64_t* lattice_steps, int32_t* macro_current,
                      int32_t* force_next, int32_t* force_last, int64_t* coupled_steps);
int fsi_ctx_set_state(fsi_ctx* ctx, int64_t lattice_steps, int32_t macro_current,
                      int32_t force_next, int32_t force_last, int64_t coupled_steps);

/* `steps` coupled steps of lbm_dt with n_substeps MPM substeps each: per step, the coupling
 * fields are cleared, each substep runs the coupling force, its spread and the MPM substep
 * (fsi_coupled_substep_tiled or fsi_coupled_substep), then contact when enabled; the force
 * for the next lattice step is assembled (base force `body_force`, host float[3], or
 * desc.base_force when NULL) and the lattice steps. Asynchronous on `stream`, no allocation
 * and no synchronisation: capturable in a CUDA graph (a graph of an even number of lattice
 * steps returns the buffers to the same parity; the host state advances at capture). */
int fsi_coupled_step(fsi_ctx* ctx, double lbm_dt, const float* body_force, int32_t n_substeps,
                     int32_t steps, void* stream);

/* The reductions behind FSISimulation.diagnostics (simulation.py:117-147) into device double
 * out[30]: [0] sum of rho over fluid cells and [1] max |u| of the current state
 * (fsi_lbm_macro_diagnostics, which also makes `macro` current, or fsi_lbm_reduce when it is;
 * [2..7] scratch), [8..29] fsi_coupled_diagnostics. */
int fsi_ctx_diagnostics(fsi_ctx* ctx, double* out, void* stream);

/* ------------------------------------------------------------- batches of scenes
 * Many independent lattices advanced together: one launch per phase covers every lattice
 * of the batch. No reference counterpart (the reference runs one scene per FSISimulation).
 * Lattice s owns cells [cell_offset, cell_offset + nx*ny*nz) of the batch's concatenated
 * per-cell arrays: populations are the [19][N_s] block at element 19 * cell_offset (in the
 * batch's storage type), force the [3][N_s] block at 3 * cell_offset, macro the [N_s][4]
 * block at cell_offset, flags and masks start at cell_offset. The offsets are the running
 * sums of the lattice sizes in order. Faces are periodic (x faces are not batched). */
typedef struct fsi_batch_lattice {
  int32_t nx, ny, nz;
  int32_t reserved;
  int64_t cell_offset;
  float s[19];          /* MRT relaxation rates, as fsi_lbm_desc.s */
  float rho0;
  float base_force[3];  /* the lattice's body force (LBMConfig.force) */
} fsi_batch_lattice;

typedef struct fsi_batch fsi_batch; /* opaque */

/* Validates the lattices (host array), copies them and the launch tiles to the device.
 * storage / arithmetic: FSI_STORAGE_* / FSI_ARITH_* for every lattice of the batch. */
int fsi_batch_create(const fsi_batch_lattice* lattices, int32_t count, int32_t storage,
                     int32_t arithmetic, fsi_batch** out);
int fsi_batch_destroy(fsi_batch* batch);
/* Total cells of the batch (the length of the concatenated per-cell arrays). */
int fsi_batch_cells(const fsi_batch* batch, int64_t* cells);

/* Launch parameters of the batched lattice step, chosen by a caller's autotuner: cells per
 * thread block (a multiple of 128, or of 256 for the fast forms; default 256) and the
 * register-cap variant 0..2 (default 1). The exact form's results do not depend on them; the
 * fast forms' may differ in the last bits (the assembler schedules each variant apart). */
int fsi_batch_tune(fsi_batch* batch, int32_t step_tile_cells, int32_t variant);

/* fsi_lbm_build_flags / fsi_lbm_init_fields / fsi_lbm_step / fsi_lbm_update_macro /
 * fsi_lbm_distribution over every lattice of the batch, with the same meaning per lattice.
 * u0: device float[count][3]. diag: NULL or device double[count][2] (sum of rho over fluid
 * cells, max |u|), zeroed here. */
int fsi_batch_lbm_flags(const fsi_batch* batch, const int32_t* solid, uint32_t* flags,
                        void* stream);
int fsi_batch_lbm_init(const fsi_batch* batch, const float* u0, const uint32_t* flags,
                       void* pops, float* macro, void* stream);
int fsi_batch_lbm_step(const fsi_batch* batch, void* pops, float* macro, const float* force,
                       const float* force_prev, const uint32_t* flags, int64_t steps_done,
                       void* stream);
int fsi_batch_lbm_macro(const fsi_batch* batch, const void* pops, const float* force,
                        const uint32_t* flags, int64_t steps_done, float* macro, double* diag,
                        void* stream);
int fsi_batch_lbm_distribution(const fsi_batch* batch, const void* pops, const uint32_t* flags,
                               int64_t steps_done, float* out, void* stream);
/* force = the lattice's base_force on fluid cells, 0 on solid cells (reset_force). */
int fsi_batch_lbm_base_force(const fsi_batch* batch, const uint32_t* flags, float* force,
                             void* stream);

/* The solid and coupling of each scene of a batch (one entry per lattice, same order).
 * Particles of all scenes live in one set of fsi_particles arrays of the batch's capacity;
 * scene s owns particles [particle_offset, particle_offset + mpm.num_particles), with
 * particle_offset a multiple of FSI_BATCH_PARTICLE_ALIGN and the ranges in scene order.
 * mpm.nx/ny/nz must equal the lattice's; mpm.dt is the MPM substep. coupling carries the
 * scene's penalty parameters and gamma_eff; dt_ratio and build_fraction are per call. The
 * MPM grid is the batch's concatenated float4 [cells] array (scene blocks at cell_offset)
 * and the dirty map one byte per 4^3 node block, scene blocks in scene order. */
#define FSI_BATCH_PARTICLE_ALIGN 256
typedef struct fsi_batch_solid {
  fsi_mpm_desc mpm;
  fsi_coupling_desc coupling;
  int64_t particle_offset;
} fsi_batch_solid;

/* Validates and installs the scenes' solids (host array of fsi_batch_count entries);
 * capacity is the particle arrays' length. Writes the dirty-map length to *dirty_blocks. */
int fsi_batch_set_solids(fsi_batch* batch, const fsi_batch_solid* solids, int64_t capacity,
                         int64_t* dirty_blocks);
/* Sets every scene's gamma_eff (host float[count]). */
int fsi_batch_set_gamma(fsi_batch* batch, const float* gamma_eff);
/* fsi_mpm_substep / fsi_coupling_forces / fsi_coupling_assemble over every scene, with the
 * same meaning per scene. counters: device fsi_coupling_counters[count]. */
int fsi_batch_mpm_substep(const fsi_batch* batch, const fsi_particles* particles, float* grid,
                          uint8_t* dirty, void* stream);
int fsi_batch_coupling_forces(const fsi_batch* batch, const fsi_particles* particles,
                              const float* macro, const uint32_t* flags, float* accum,
                              float* valid_weight, int32_t* coupling_mask, void* counters,
                              float dt_ratio, int32_t build_fraction, void* stream);
int fsi_batch_coupling_assemble(const fsi_batch* batch, const uint32_t* flags, int32_t mode,
                                float* accum, const float* macro, float* force, float* ib_force,
                                void* counters, void* stream);

/* Device arrays of a scene batch's coupled state, for fsi_batch_run_persistent. */
typedef struct fsi_batch_state {
  void* pops;             /* populations, the batch's storage form */
  float* macro;           /* float[cells][4] */
  float* force[2];        /* the two force buffers, float[3][cells] scene blocks each */
  const uint32_t* flags;  /* from fsi_batch_lbm_flags */
  float* accum;           /* float[cells][4] coupling accumulator */
  float* ib_force;        /* float[3][cells] scene blocks, or NULL */
  float* valid_weight;    /* float[capacity] */
  int32_t* coupling_mask; /* int32[capacity] */
  void* counters;         /* fsi_coupling_counters[count] */
  float* grid;            /* float4[cells], all-zero between substeps */
  uint8_t* dirty;         /* dirty map of fsi_batch_set_solids */
  uint32_t* sync;         /* one device word for the grid barrier (zeroed by each call) */
  int32_t* error;         /* one device word: left 0, or set to FSI_ERR_TIMEOUT when a
                             barrier wait gave up (the caller clears it) */
} fsi_batch_state;

/* `steps` coupled steps of every scene in one persistent cooperative launch (as many
 * 256-thread blocks as are resident at once, grid-wide barriers between phases): per step
 * the rho / u refresh and accumulator zeroing, `substeps` x (fsi_batch_coupling_forces with
 * build_fraction on the first substep, fsi_batch_mpm_substep), fsi_batch_coupling_assemble
 * with assemble_mode into force[1 - prev], and the lattice step (parity of steps_done) with
 * that force; then prev flips. prev_force is the buffer of the step before the first;
 * macro_fresh says whether rho / u of the current state are already in macro. Every
 * barrier wait is bounded by wait_cycles SM clock cycles (0: 2^31, about a second): a launch
 * that gives up sets *error and ends, its state then undefined.
 * Each scene's result is that of the per-phase calls. No reference counterpart: the
 * reference runs one scene per simulation (fsi/simulation.py:12-153). */
int fsi_batch_run_persistent(const fsi_batch* batch, const fsi_particles* particles,
                             const fsi_batch_state* state, int64_t steps_done, int32_t steps,
                             int32_t substeps, float dt_ratio, int32_t build_fraction,
                             int32_t assemble_mode, int32_t prev_force, int32_t macro_fresh,
                             int64_t wait_cycles, void* stream);

/* ------------------------------------------------------------ learned closure
 * A per-cell MLP (656 -> 64 -> 64 -> 64 -> 19, GELU, BF16 weights, FP32 accumulation) that
 * corrects the post-stream populations of a lattice run on a grid 2x coarser than the one it
 * was trained on, on the tcgen05 tensor cores. No reference counterpart. Lattices must use
 * FP32 population storage. Features of a cell: for each of its 27 neighbours (periodic wrap,
 * offsets (dx, dy, dz) in {-1,0,1}^3 with dz fastest) the 19 populations as
 * (f_q - w_q rho0) * pop_scale, the occupancy (solid fraction, or 1 solid) and the
 * force * force_scale:
 * 27 * 23 = 621 values, neighbour o in columns [24 o, 24 o + 23), column 24 o + 23 and columns
 * 648..655 zero: 656 columns. */
#define FSI_CLOSURE_FEATURES 656

/* Feature rows (BF16 [m][656]) of the cells listed in `cells` (device int32[m]). The
 * occupancy feature is solid_fraction[cell] (device float[N], the share of a coarse cell's
 * fine children that are solid) when given, else 1 for solid and 0 for fluid cells; the
 * inference entries below take the same argument. */
int fsi_closure_features(const fsi_lbm_desc* desc, const float* pops, const uint32_t* flags,
                         const float* force, const float* solid_fraction, int64_t steps_done,
                         const int32_t* cells, int32_t m, float pop_scale, float force_scale,
                         void* x, void* stream);

/* C = A B^T with BF16 K-major operands A [m][lda], B [n][ldb] (row-major, 16-byte aligned,
 * lda and ldb multiples of 8) on the tensor cores, K split into k_chunk pieces over the grid,
 * and one epilogue:
 *   0  C[r][c] = acc                        (FP32, ldc)
 *   1  C[r][c] += acc atomically            (FP32, ldc; for split-K weight gradients)
 *   2  z = acc + bias[c]; zout[r][c] = z (if not NULL); h[r][c] = ht[c][r] = gelu(z) (BF16)
 *   3  h[r][c] = ht[c][r] = acc * gelu'(zin[r][c])                                (BF16)
 * (h, zout, zin are [m][n]; ht is [n][ldht] or NULL.) err: device int, set non-zero if a
 * wait on the tensor cores timed out. */
typedef struct fsi_closure_gemm_desc {
  const void* a;
  const void* b;
  int32_t lda, ldb;
  int32_t m, n, k, k_chunk;
  int32_t mode;
  int32_t ldc;
  float* c;
  const float* bias;
  void* h;
  void* ht;
  int32_t ldht;
  int32_t reserved;
  float* zout;
  const float* zin;
  int32_t* err;
} fsi_closure_gemm_desc;
int fsi_closure_gemm(const fsi_closure_gemm_desc* desc, void* stream);

/* Network of the fused inference: BF16 w1 [64][656], w2 [64][64], w3 [64][64], w4 [32][64]
 * (rows 19..31 zero), FP32 bias = b1[64] b2[64] b3[64] b4[32]; correction = y / out_scale. */
typedef struct fsi_closure_weights {
  const void* w1;
  const void* w2;
  const void* w3;
  const void* w4;
  const float* bias;
  float pop_scale;
  float force_scale;
  float out_scale;
  int32_t reserved;
} fsi_closure_weights;

/* Bytes of the scratch `rows` buffer fsi_closure_infer needs for this lattice (the BF16
 * feature rows of every cell on a lattice padded to whole inference columns), or -1. */
int64_t fsi_closure_rows_bytes(const fsi_lbm_desc* desc);
/* Fused inference over every cell: the cells' feature rows written to `rows` (16-byte
 * aligned, fsi_closure_rows_bytes bytes), then layer 1 as a 3x3x3 convolution and the four
 * layers on the tensor cores with the weights resident in shared memory; corrections
 * corr [19][N] (0 on solid cells). Network: BF16 w1 [64][656]. */
int fsi_closure_infer(const fsi_lbm_desc* desc, const float* pops, const uint32_t* flags,
                      const float* force, const float* solid_fraction, int64_t steps_done,
                      const fsi_closure_weights* weights,
                      void* rows, float* corr, int32_t* err, void* stream);
/* fsi_closure_infer followed by fsi_closure_apply in one pass: each fluid cell's
 * mass-conserving correction is added to its populations in place (the arithmetic of
 * fsi_closure_apply), without a correction array. */
int fsi_closure_infer_apply(const fsi_lbm_desc* desc, float* pops, const uint32_t* flags,
                            const float* force, const float* solid_fraction, int64_t steps_done,
                            const fsi_closure_weights* weights, void* rows, int32_t* err,
                            void* stream);
/* f_q += corr_q - w_q sum_p corr_p on fluid cells (moves no mass). */
int fsi_closure_apply(const fsi_lbm_desc* desc, float* pops, const uint32_t* flags,
                      int64_t steps_done, const float* corr, void* stream);
/* Mean post-stream populations of the fluid children of each coarse cell, out [Nc][19]. */
int fsi_closure_restrict(const fsi_lbm_desc* fine, const float* pops, const uint32_t* flags,
                         int64_t steps_done, const fsi_lbm_desc* coarse, float* out,
                         void* stream);
/* Training: mean-square loss of y [m][32] + b4 against target [m][19], its gradient dy
 * (BF16 [m][32]) and transpose dyt ([32][ldt]); loss (device double) accumulates. */
int fsi_closure_loss(const float* y, const float* target, const float* b4, int32_t m, void* dy,
                     void* dyt, int32_t ldt, double* loss, void* stream);
/* out[c] += sum_r g[r][c] for BF16 g [m][n]. */
int fsi_closure_colsum(const void* g, int32_t m, int32_t n, float* out, void* stream);
/* One Adam step (bias-corrected) of n parameters. */
int fsi_closure_adam(float* params, const float* grads, float* m, float* v, int64_t n, float lr,
                     float beta1, float beta2, float eps, int32_t step, void* stream);

/* Self-test of the bounded mbarrier waits of the tensor-core kernels (no reference
 * counterpart; a failure-detection check that faults nothing). One CTA waits on a barrier that
 * nothing arrives on: out[0] = 0 when the plain wait gave up after its clock limit (about one
 * second) and set *err = 7; out[1] = 0 when a second role's abortable wait returned on the
 * first role's abort flag without setting its own code (8). err (zeroed by the caller) and
 * out are device int32 arrays of 1 and 2 elements. */
int fsi_selftest_wait_limit(int32_t* err, int32_t* out, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* FSI_GB300_H */
