// One coupled scene behind a context: LBMMpmCoupler.step (fsi/coupling.py:135-173) as one C
// call for hosts without the Python package.
//
// The context holds the scene's descriptors, the caller's buffer pointers, the lattice
// bookkeeping of LBMSolver3D (steps taken, which force buffer the next and the last step
// use, whether rho/u are current) and its own scratch: the MPM grid and block map (atomic
// scatter) or the sorted-scatter workspace. fsi_coupled_step issues the entry points of this
// library in the order of the Python coupler, so the two paths launch the same kernels with
// the same arguments.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "fsi_common.cuh"

struct fsi_ctx {
  fsi_scene_desc d{};
  fsi_scene_buffers b{};
  // scratch owned by the context
  float* grid = nullptr;
  uint8_t* dirty = nullptr;
  void* workspace = nullptr;
  int64_t workspace_bytes = 0;
  // lattice bookkeeping (LBMSolver3D._steps_done / _macro_fresh / _fcur / _fprev)
  int64_t lattice_steps = 0;
  bool macro_current = true;
  int force_next = 0;
  int force_last = -1;
  int64_t coupled_steps = 0;
  bool ib_written = false;
};

namespace fsi {
namespace {

long long cells_of(const fsi_lbm_desc& l) { return (long long)l.nx * l.ny * l.nz; }

int cuda_status(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return FSI_OK;
  set_error("%s: %s", what, cudaGetErrorString(e));
  return FSI_ERR_CUDA;
}

// _effective_gamma of coupling.py:321-330 in float32.
float ramped_gamma(const fsi_scene_desc& d, int64_t coupled_step) {
  float g = d.gamma;
  if (d.gamma_ramp_steps > 0) {
    const float r = ((float)coupled_step + 1.0f) / (float)d.gamma_ramp_steps;
    g = g * std::min(1.0f, r);
  }
  return g;
}

// The force buffer a force update may overwrite without losing the force of the last step
// (LBMSolver3D._target_force_buffer).
int writable_force(fsi_ctx* c) {
  if (c->force_next == c->force_last) c->force_next = 1 - c->force_next;
  return c->force_next;
}

// update_macro when rho, u are stale (LBMSolver3D._ensure_macro).
int ensure_macro(fsi_ctx* c, void* stream) {
  if (c->macro_current) return FSI_OK;
  if (int e = fsi_lbm_update_macro(&c->d.lbm, c->b.pops, c->b.force[c->force_last], c->b.flags,
                                   c->lattice_steps, c->b.macro, stream))
    return e;
  c->macro_current = true;
  return FSI_OK;
}

// LBMSolver3D.step (lbm3d.py:427-433): the force of force_next, rho/u from macro when current
// and otherwise recomputed from the populations and the last step's force.
int lattice_step(fsi_ctx* c, void* stream) {
  const float* force = c->b.force[c->force_next];
  const float* prev = nullptr;
  if (!c->macro_current) prev = c->force_last == c->force_next ? force : c->b.force[c->force_last];
  if (int e = fsi_lbm_step(&c->d.lbm, c->b.pops, c->b.macro, force, prev, c->b.flags,
                           c->lattice_steps, stream))
    return e;
  c->lattice_steps += 1;
  c->force_last = c->force_next;
  c->macro_current = false;
  return FSI_OK;
}

// clear_coupling_fields + clear_particle_diagnostics (coupling.py:198-224).
int clear_coupling_fields(fsi_ctx* c, cudaStream_t s) {
  const long long n = cells_of(c->d.lbm);
  const long long cap = c->b.particles.capacity;
  if (int e = cuda_status(cudaMemsetAsync(c->b.accum, 0, sizeof(float) * 4 * n, s), "accum"))
    return e;
  if (c->ib_written) {  // the IB force field stays zero while nothing writes it
    if (int e = cuda_status(cudaMemsetAsync(c->b.ib_force, 0, sizeof(float) * 3 * n, s), "ib"))
      return e;
    c->ib_written = c->d.immersed_boundary_enabled != 0;
  }
  if (int e = cuda_status(cudaMemsetAsync(c->b.counters, 0, sizeof(fsi_coupling_counters), s),
                          "counters"))
    return e;
  if (int e = cuda_status(cudaMemsetAsync(c->b.valid_weight, 0, sizeof(float) * cap, s), "valid"))
    return e;
  if (int e = cuda_status(cudaMemsetAsync(c->b.coupling_mask, 0, sizeof(int32_t) * cap, s), "mask"))
    return e;
  if (c->b.contact_mask)
    if (int e = cuda_status(cudaMemsetAsync(c->b.contact_mask, 0, sizeof(int32_t) * cap, s),
                            "contact mask"))
      return e;
  return FSI_OK;
}

// MPMSolver3D.clear_particle_force: the forces of the live particles.
int clear_particle_force(fsi_ctx* c, cudaStream_t s) {
  const long long cap = c->b.particles.capacity;
  const size_t live = sizeof(float) * (size_t)c->d.mpm.num_particles;
  for (int a = 0; a < 3; ++a)
    if (int e = cuda_status(cudaMemsetAsync(c->b.particles.force + a * cap, 0, live, s), "force"))
      return e;
  return FSI_OK;
}

int one_step(fsi_ctx* c, double lbm_dt, const float* body_force, int n_substeps, void* stream) {
  cudaStream_t s = as_stream(stream);
  fsi_scene_desc& d = c->d;
  const bool enabled = d.coupling_enabled != 0;
  if (int e = clear_coupling_fields(c, s)) return e;
  if (enabled) {
    if (int e = ensure_macro(c, stream)) return e;  // the coupling reads rho, u
  }
  const double mpm_dt = lbm_dt / (double)n_substeps;
  const double dt_ratio = mpm_dt / lbm_dt;
  d.mpm.dt = (float)mpm_dt;
  d.coupling.gamma_eff = ramped_gamma(d, c->coupled_steps);
  d.coupling.dt_ratio = (float)dt_ratio;
  const fsi_particles* P = &c->b.particles;
  for (int sub = 0; sub < n_substeps; ++sub) {
    if (enabled) {
      d.coupling.build_fraction = (sub == 0 && d.build_solid_fraction) ? 1 : 0;
      int e;
      if (d.p2g_mode == FSI_P2G_SORTED)
        e = fsi_coupled_substep(&d.coupling, &d.mpm, P, c->b.macro, c->b.flags, c->b.accum,
                                c->b.valid_weight, c->b.coupling_mask, c->b.counters, c->grid,
                                c->workspace, c->workspace_bytes, stream);
      else
        e = fsi_coupled_substep_tiled(&d.coupling, &d.mpm, P, c->b.macro, c->b.flags,
                                      c->b.accum, c->b.valid_weight, c->b.coupling_mask,
                                      c->b.counters, c->grid, c->dirty, stream);
      if (e) return e;
    } else {
      if (int e = clear_particle_force(c, s)) return e;
      int e;
      if (d.p2g_mode == FSI_P2G_SORTED)
        e = fsi_mpm_substep_sorted(&d.mpm, P, c->grid, c->workspace, c->workspace_bytes, stream);
      else
        e = fsi_mpm_substep(&d.mpm, P, c->grid, c->dirty, stream);
      if (e) return e;
    }
    if (d.contact_enabled) {
      if (int e = fsi_contact(&d.coupling, &d.mpm, P, c->b.accum, c->b.flags, c->b.contact_mask,
                              c->b.counters, stream))
        return e;
    }
  }
  int mode = 0;
  if (enabled && d.build_solid_fraction) mode |= FSI_ASSEMBLE_CLAMP_FRACTION;
  if (enabled) mode |= FSI_ASSEMBLE_COUPLING;
  const float* macro = nullptr;
  if (d.immersed_boundary_enabled) {
    mode |= FSI_ASSEMBLE_IB;
    c->ib_written = true;
    if (int e = ensure_macro(c, stream)) return e;
    macro = c->b.macro;
  }
  const float* base = body_force ? body_force : d.base_force;
  const int dst = writable_force(c);
  if (int e = fsi_coupling_assemble(&d.coupling, &d.lbm, c->b.flags, base, mode, c->b.accum,
                                    macro, c->b.force[dst], c->b.ib_force, c->b.counters, stream))
    return e;
  if (int e = lattice_step(c, stream)) return e;
  if (enabled) c->coupled_steps += 1;
  return FSI_OK;
}

}  // namespace
}  // namespace fsi

using namespace fsi;

extern "C" int fsi_ctx_create(const fsi_scene_desc* desc, const fsi_scene_buffers* buffers,
                              fsi_ctx** out) {
  FSI_REQUIRE(desc && buffers && out, "NULL argument");
  *out = nullptr;
  const fsi_scene_buffers& b = *buffers;
  const fsi_scene_desc& d = *desc;
  FSI_REQUIRE(d.lbm.nx > 0 && d.lbm.ny > 0 && d.lbm.nz > 0, "empty lattice");
  FSI_REQUIRE(d.mpm.nx == d.lbm.nx && d.mpm.ny == d.lbm.ny && d.mpm.nz == d.lbm.nz,
              "the MPM grid %dx%dx%d must coincide with the lattice %dx%dx%d", d.mpm.nx,
              d.mpm.ny, d.mpm.nz, d.lbm.nx, d.lbm.ny, d.lbm.nz);
  FSI_REQUIRE(d.p2g_mode == FSI_P2G_ATOMIC || d.p2g_mode == FSI_P2G_SORTED, "unknown p2g_mode %d",
              d.p2g_mode);
  FSI_REQUIRE(b.pops && b.macro && b.force[0] && b.force[1] && b.flags, "NULL lattice buffer");
  FSI_REQUIRE(b.force[0] != b.force[1], "the two force buffers must differ");
  FSI_REQUIRE(b.accum && b.valid_weight && b.coupling_mask && b.counters, "NULL coupling buffer");
  FSI_REQUIRE(!d.immersed_boundary_enabled || b.ib_force, "the immersed boundary needs ib_force");
  FSI_REQUIRE(!d.contact_enabled || b.contact_mask, "contact needs contact_mask");
  FSI_REQUIRE(b.particles.x && b.particles.v && b.particles.C && b.particles.F &&
                  b.particles.mass && b.particles.volume && b.particles.active &&
                  b.particles.force,
              "NULL particle array");
  FSI_REQUIRE(d.mpm.num_particles >= 0 && d.mpm.num_particles <= b.particles.capacity,
              "num_particles %d outside [0, capacity %lld]", d.mpm.num_particles,
              (long long)b.particles.capacity);
  fsi_ctx* c = new fsi_ctx();
  c->d = d;
  c->b = b;
  const long long n = cells_of(d.lbm);
  int err = FSI_OK;
  if (d.p2g_mode == FSI_P2G_SORTED) {
    err = fsi_mpm_workspace_bytes(&d.mpm, b.particles.capacity, &c->workspace_bytes);
    if (!err) err = cuda_status(cudaMalloc(&c->workspace, c->workspace_bytes), "workspace");
    if (!err) err = cuda_status(cudaMemset(c->workspace, 0, c->workspace_bytes), "workspace");
  } else {
    const long long blocks = (long long)((d.mpm.nx + 3) / 4) * ((d.mpm.ny + 3) / 4) * ((d.mpm.nz + 3) / 4);
    err = cuda_status(cudaMalloc(&c->dirty, blocks), "dirty");
    if (!err) err = cuda_status(cudaMemset(c->dirty, 0, blocks), "dirty");
  }
  if (!err) err = cuda_status(cudaMalloc(&c->grid, sizeof(float) * 4 * n), "grid");
  if (!err) err = cuda_status(cudaMemset(c->grid, 0, sizeof(float) * 4 * n), "grid");
  if (!err) err = cuda_status(cudaDeviceSynchronize(), "fsi_ctx_create");
  if (err) {
    fsi_ctx_destroy(c);
    return err;
  }
  *out = c;
  return FSI_OK;
}

extern "C" int fsi_ctx_destroy(fsi_ctx* c) {
  if (!c) return FSI_OK;
  cudaFree(c->grid);
  cudaFree(c->dirty);
  cudaFree(c->workspace);
  delete c;
  return FSI_OK;
}

extern "C" int fsi_ctx_get_state(const fsi_ctx* c, int64_t* lattice_steps, int32_t* macro_current,
                                 int32_t* force_next, int32_t* force_last, int64_t* coupled_steps) {
  FSI_REQUIRE(c, "NULL context");
  if (lattice_steps) *lattice_steps = c->lattice_steps;
  if (macro_current) *macro_current = c->macro_current ? 1 : 0;
  if (force_next) *force_next = c->force_next;
  if (force_last) *force_last = c->force_last;
  if (coupled_steps) *coupled_steps = c->coupled_steps;
  return FSI_OK;
}

extern "C" int fsi_ctx_set_state(fsi_ctx* c, int64_t lattice_steps, int32_t macro_current,
                                 int32_t force_next, int32_t force_last, int64_t coupled_steps) {
  FSI_REQUIRE(c, "NULL context");
  FSI_REQUIRE(lattice_steps >= 0 && coupled_steps >= 0, "negative step count");
  FSI_REQUIRE(force_next == 0 || force_next == 1, "force_next must be 0 or 1");
  FSI_REQUIRE(force_last >= -1 && force_last <= 1, "force_last must be -1, 0 or 1");
  FSI_REQUIRE(macro_current || force_last >= 0,
              "stale rho/u need the force of the last step (force_last)");
  c->lattice_steps = lattice_steps;
  c->macro_current = macro_current != 0;
  c->force_next = force_next;
  c->force_last = force_last;
  c->coupled_steps = coupled_steps;
  return FSI_OK;
}

extern "C" int fsi_coupled_step(fsi_ctx* c, double lbm_dt, const float* body_force,
                                int32_t n_substeps, int32_t steps, void* stream) {
  FSI_REQUIRE(c, "NULL context");
  FSI_REQUIRE(lbm_dt > 0.0 && std::isfinite(lbm_dt), "lbm_dt must be positive.");
  FSI_REQUIRE(n_substeps > 0, "n_substeps must be positive");
  FSI_REQUIRE(steps >= 0, "steps must be non-negative");
  for (int i = 0; i < steps; ++i)
    if (int e = one_step(c, lbm_dt, body_force, n_substeps, stream)) return e;
  return FSI_OK;
}

extern "C" int fsi_ctx_diagnostics(fsi_ctx* c, double* out, void* stream) {
  FSI_REQUIRE(c && out, "NULL argument");
  if (c->macro_current) {
    if (int e = fsi_lbm_reduce(&c->d.lbm, c->b.macro, c->b.force[c->force_next], c->b.flags, out,
                               stream))
      return e;
  } else {
    if (int e = fsi_lbm_macro_diagnostics(&c->d.lbm, c->b.pops, c->b.force[c->force_last],
                                          c->b.flags, c->lattice_steps, c->b.macro, out, stream))
      return e;
    c->macro_current = true;
  }
  return fsi_coupled_diagnostics(&c->d.mpm, &c->b.particles, &c->d.lbm, c->b.accum, c->b.flags,
                                 c->b.counters, out + 8, stream);
}
