// CPU oracle for the coupled LBM-MPM timestep of lizhuoh9/taichi-mpm-lbm.
//
// TEST INFRASTRUCTURE ONLY. This file is a literal restatement of the
// reference's Taichi kernels in plain C++ (templated on float / double) so
// that the CUDA implementation can be checked against it. It is never linked
// into, loaded by, or called from the product library; only tests/, the smoke
// check and bench.py's CPU-baseline leg use it.
//
// Arithmetic follows the reference source order term by term (sequential sums
// in index order, no fused multiply-add: build with -ffp-contract=off), so the
// float instantiation reproduces what the reference computes in FP32 up to the
// reference runtime's own freedom (Taichi fast-math, atomic ordering).
//
// Layouts are the reference's numpy layouts (C order):
//   f, F      [nx, ny, nz, 19]      rho [nx, ny, nz]     v, force [nx, ny, nz, 3]
//   solid     [nx, ny, nz] int32    particles x, v, f_p [P, 3]; C, F [P, 3, 3]
//   grid_v    [nx, ny, nz, 3]       grid_m [nx, ny, nz]
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr int Q = 19;

// D3Q19 velocity ordering, fsi/lbm3d.py:221-239.
const int E[Q][3] = {{0, 0, 0},  {1, 0, 0},   {-1, 0, 0}, {0, 1, 0},  {0, -1, 0},
                     {0, 0, 1},  {0, 0, -1},  {1, 1, 0},  {-1, -1, 0}, {1, -1, 0},
                     {-1, 1, 0}, {1, 0, 1},   {-1, 0, -1}, {1, 0, -1}, {-1, 0, 1},
                     {0, 1, 1},  {0, -1, -1}, {0, 1, -1}, {0, -1, 1}};
// Opposite directions, fsi/lbm3d.py:171-174.
const int LR[Q] = {0, 2, 1, 4, 3, 6, 5, 8, 7, 10, 9, 12, 11, 14, 13, 16, 15, 18, 17};

inline int nthreads_or_default(int n) { return n > 0 ? n : 1; }

template <class T>
struct Lattice {
  int nx, ny, nz;
  const T* M;     // [19][19] MRT matrix (fsi/lbm3d.py:30-54)
  const T* invM;  // [19][19] numpy inverse of M in float32, widened (lbm3d.py:170)
  const T* S;     // [19] relaxation rates (lbm3d.py:141-168)
  const T* w;     // [19] lattice weights (lbm3d.py:244-248)
  long cell(int i, int j, int k) const { return ((long)i * ny + j) * nz + k; }
  long ncell() const { return (long)nx * ny * nz; }
};

template <class T>
inline T dot3(const T a[3], const T b[3]) {
  // Taichi Vector.dot: elementwise product then sequential sum.
  T s = a[0] * b[0];
  s = s + a[1] * b[1];
  s = s + a[2] * b[2];
  return s;
}

// feq, fsi/lbm3d.py:250-254.
template <class T>
inline T feq(const Lattice<T>& L, int q, T rho, const T u[3]) {
  T e[3] = {(T)E[q][0], (T)E[q][1], (T)E[q][2]};
  T eu = dot3(e, u);
  T uv = dot3(u, u);
  T inner = (T)1.0 + (T)3.0 * eu;
  inner = inner + ((T)4.5 * eu) * eu;
  inner = inner - (T)1.5 * uv;
  return (L.w[q] * rho) * inner;
}

// meq_vec, fsi/lbm3d.py:285-312.
template <class T>
inline T meq_vec(int m, T rho, const T u[3]) {
  T out = 0;
  if (m == 0) out = rho;
  if (m == 1) out = dot3(u, u);
  if (m == 3) out = u[0];
  if (m == 5) out = u[1];
  if (m == 7) out = u[2];
  if (m == 9) out = (((T)2.0 * u[0]) * u[0] - u[1] * u[1]) - u[2] * u[2];
  if (m == 11) out = u[1] * u[1] - u[2] * u[2];
  if (m == 13) out = u[0] * u[1];
  if (m == 14) out = u[1] * u[2];
  if (m == 15) out = u[0] * u[2];
  return out;
}

// guo_force, fsi/lbm3d.py:276-283.
template <class T>
inline T guo_force(const Lattice<T>& L, int m, const T u[3], const T G[3]) {
  T out = 0;
  for (int q = 0; q < Q; ++q) {
    T e[3] = {(T)E[q][0], (T)E[q][1], (T)E[q][2]};
    T emu[3] = {e[0] - u[0], e[1] - u[1], e[2] - u[2]};
    T a = dot3(emu, G);
    T b = dot3(e, u) * dot3(e, G);
    out = out + (L.w[q] * (a + b)) * L.M[m * Q + q];
  }
  return out;
}

// collide, fsi/lbm3d.py:314-333 (fluid cells only; writes f from F).
template <class T>
void collide(const Lattice<T>& L, T* f, const T* F, const T* rho, const T* v, const T* force,
             const int32_t* solid, int nthreads) {
  const long n = L.ncell();
#pragma omp parallel for schedule(static) num_threads(nthreads_or_default(nthreads))
  for (long c = 0; c < n; ++c) {
    if (solid[c] != 0) continue;
    const T* Fc = F + c * Q;
    T u[3] = {v[3 * c], v[3 * c + 1], v[3 * c + 2]};
    T G[3] = {force[3 * c], force[3 * c + 1], force[3 * c + 2]};
    T mom[Q];
    for (int m = 0; m < Q; ++m) {
      T mv = 0;
      for (int q = 0; q < Q; ++q) mv = mv + L.M[m * Q + q] * Fc[q];
      T meq = meq_vec(m, rho[c], u);
      mv = mv - L.S[m] * (mv - meq);
      mv = mv + ((T)1.0 - (T)0.5 * L.S[m]) * guo_force(L, m, u, G);
      mom[m] = mv;
    }
    for (int q = 0; q < Q; ++q) {
      T acc = 0;
      for (int m = 0; m < Q; ++m) acc = acc + L.invM[q * Q + m] * mom[m];
      f[c * Q + q] = acc;
    }
  }
}

// stream + periodic_index, fsi/lbm3d.py:335-361.
template <class T>
void stream(const Lattice<T>& L, const T* f, T* F, const int32_t* solid, int nthreads) {
#pragma omp parallel for schedule(static) num_threads(nthreads_or_default(nthreads))
  for (int i = 0; i < L.nx; ++i)
    for (int j = 0; j < L.ny; ++j)
      for (int k = 0; k < L.nz; ++k) {
        long c = L.cell(i, j, k);
        if (solid[c] != 0) continue;
        for (int q = 0; q < Q; ++q) {
          int ti = i + E[q][0], tj = j + E[q][1], tk = k + E[q][2];
          if (ti < 0) ti = L.nx - 1;
          if (ti > L.nx - 1) ti = 0;
          if (tj < 0) tj = L.ny - 1;
          if (tj > L.ny - 1) tj = 0;
          if (tk < 0) tk = L.nz - 1;
          if (tk > L.nz - 1) tk = 0;
          long t = L.cell(ti, tj, tk);
          if (solid[t] == 0)
            F[t * Q + q] = f[c * Q + q];
          else
            F[c * Q + LR[q]] = f[c * Q + q];
        }
      }
}

// apply_boundary, fsi/lbm3d.py:363-407. mode 1 = pressure, 2 = velocity (in place, in q
// order, as the reference), 3 = velocity with every population read from before the update
// (an extension with no reference counterpart).
template <class T>
void apply_boundary_face(const Lattice<T>& L, T* F, const T* v, const int32_t* solid, int xi,
                         int xin, int mode, T bc_rho, const T bc_vel[3], T rho0) {
  if (mode == 0) return;
  for (int j = 0; j < L.ny; ++j)
    for (int k = 0; k < L.nz; ++k) {
      long c = L.cell(xi, j, k);
      if (solid[c] != 0) continue;
      if (mode == 1) {
        long ci = L.cell(xin, j, k);
        const T* uu = solid[ci] > 0 ? v + 3 * ci : v + 3 * c;
        T u[3] = {uu[0], uu[1], uu[2]};
        for (int q = 0; q < Q; ++q) F[c * Q + q] = feq(L, q, bc_rho, u);
      } else if (mode == 2) {
        for (int q = 0; q < Q; ++q) {
          int o = LR[q];
          T val = feq(L, o, rho0, bc_vel) - F[c * Q + o];
          val = val + feq(L, q, rho0, bc_vel);
          F[c * Q + q] = val;
        }
      } else {
        T old[Q];
        for (int q = 0; q < Q; ++q) old[q] = F[c * Q + q];
        for (int q = 0; q < Q; ++q) {
          int o = LR[q];
          T val = feq(L, o, rho0, bc_vel) - old[o];
          val = val + feq(L, q, rho0, bc_vel);
          F[c * Q + q] = val;
        }
      }
    }
}

// update_macro, fsi/lbm3d.py:409-425.
template <class T>
void update_macro(const Lattice<T>& L, T* f, const T* F, T* rho, T* v, const T* force,
                  const int32_t* solid, T rho0, int nthreads) {
  const long n = L.ncell();
#pragma omp parallel for schedule(static) num_threads(nthreads_or_default(nthreads))
  for (long c = 0; c < n; ++c) {
    if (solid[c] == 0) {
      T r = 0;
      T u[3] = {0, 0, 0};
      for (int q = 0; q < Q; ++q) {
        T fq = F[c * Q + q];
        f[c * Q + q] = fq;
        r = r + fq;
        for (int a = 0; a < 3; ++a) u[a] = u[a] + (T)E[q][a] * fq;
      }
      for (int a = 0; a < 3; ++a) u[a] = u[a] / r;
      for (int a = 0; a < 3; ++a) u[a] = u[a] + (force[3 * c + a] * (T)0.5) / r;
      rho[c] = r;
      for (int a = 0; a < 3; ++a) v[3 * c + a] = u[a];
    } else {
      rho[c] = rho0;
      v[3 * c] = v[3 * c + 1] = v[3 * c + 2] = 0;
    }
  }
}

// ---------------------------------------------------------------- MPM -----

template <class T>
struct Particles {
  int n;
  T* x;        // [P,3]
  T* v;        // [P,3]
  T* C;        // [P,9]
  T* Fd;       // [P,9]
  const T* mass;
  const T* vol;
  const int32_t* active;
  T* fp;       // [P,3] particle_force
  const T* mu_p;   // per-particle Lame parameters or nullptr
  const T* lam_p;
};

template <class T>
struct Grid {
  int nx, ny, nz;
  T* gv;  // [N,3]
  T* gm;  // [N]
  long cell(int i, int j, int k) const { return ((long)i * ny + j) * nz + k; }
  bool inside(int i, int j, int k) const {
    return 0 <= i && i < nx && 0 <= j && j < ny && 0 <= k && k < nz;
  }
};

// _weights, fsi/mpm3d.py:227-232 (also coupling.py:314-319).
template <class T>
inline void bspline(T fx, T w[3]) {
  T a = (T)1.5 - fx;
  T b = fx - (T)1.0;
  T c = fx - (T)0.5;
  w[0] = (T)0.5 * (a * a);
  w[1] = (T)0.75 - b * b;
  w[2] = (T)0.5 * (c * c);
}

// base = trunc(x * inv_dx - 0.5), fx = x * inv_dx - base (mpm3d.py:239-241).
template <class T>
inline void base_fx(const T x[3], T inv_dx, int base[3], T fx[3]) {
  for (int a = 0; a < 3; ++a) {
    T g = x[a] * inv_dx;
    base[a] = (int)(g - (T)0.5);
    fx[a] = x[a] * inv_dx - (T)base[a];
  }
}

template <class T>
inline void matmul3(const T A[9], const T B[9], T out[9]) {
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) {
      T s = A[3 * a] * B[b];
      s = s + A[3 * a + 1] * B[3 + b];
      s = s + A[3 * a + 2] * B[6 + b];
      out[3 * a + b] = s;
    }
}

template <class T>
inline T det3(const T a[9]) {
  // Cofactor expansion along the first column.
  T t0 = a[4] * a[8] - a[7] * a[5];
  T t1 = a[1] * a[8] - a[7] * a[2];
  T t2 = a[1] * a[5] - a[4] * a[2];
  T d = a[0] * t0 - a[3] * t1;
  d = d + a[6] * t2;
  return d;
}

// Rotation R of the polar decomposition F = R S, computed in double precision
// by the one-sided Jacobi SVD (Hestenes 1958) of F: orthogonalise the columns
// of A = F V by plane rotations, then R = U V^T with U = A / |A| column-wise.
// The reference takes R = U V^T from ti.svd (mpm3d.py:245-246); for det F > 0
// this rotation is unique, so any accurate method agrees with it to rounding.
// For det F <= 0 the sign of the column with the smallest norm is flipped to
// return a proper rotation, which is the convention of 3x3 SVDs that keep
// det U = det V = +1.
inline void polar_rotation_f64(const double F[9], double R[9]) {
  double A[9], V[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  for (int i = 0; i < 9; ++i) A[i] = F[i];
  for (int sweep = 0; sweep < 60; ++sweep) {
    double off = 0.0;
    for (int p = 0; p < 2; ++p)
      for (int q = p + 1; q < 3; ++q) {
        double alpha = 0, beta = 0, gamma = 0;
        for (int r = 0; r < 3; ++r) {
          alpha += A[3 * r + p] * A[3 * r + p];
          beta += A[3 * r + q] * A[3 * r + q];
          gamma += A[3 * r + p] * A[3 * r + q];
        }
        if (gamma == 0.0) continue;
        off = std::fmax(off, std::fabs(gamma) / std::sqrt(alpha * beta));
        double zeta = (beta - alpha) / (2.0 * gamma);
        double t = (zeta >= 0 ? 1.0 : -1.0) / (std::fabs(zeta) + std::sqrt(1.0 + zeta * zeta));
        double c = 1.0 / std::sqrt(1.0 + t * t), s = c * t;
        for (int r = 0; r < 3; ++r) {
          double ap = A[3 * r + p], aq = A[3 * r + q];
          A[3 * r + p] = c * ap - s * aq;
          A[3 * r + q] = s * ap + c * aq;
          double vp = V[3 * r + p], vq = V[3 * r + q];
          V[3 * r + p] = c * vp - s * vq;
          V[3 * r + q] = s * vp + c * vq;
        }
      }
    if (off < 1e-15) break;
  }
  double nrm[3];
  for (int c = 0; c < 3; ++c)
    nrm[c] = std::sqrt(A[c] * A[c] + A[3 + c] * A[3 + c] + A[6 + c] * A[6 + c]);
  double U[9];
  for (int c = 0; c < 3; ++c)
    for (int r = 0; r < 3; ++r) U[3 * r + c] = nrm[c] > 0 ? A[3 * r + c] / nrm[c] : (r == c ? 1.0 : 0.0);
  double detF = F[0] * (F[4] * F[8] - F[7] * F[5]) - F[3] * (F[1] * F[8] - F[7] * F[2]) +
                F[6] * (F[1] * F[5] - F[4] * F[2]);
  double detU = U[0] * (U[4] * U[8] - U[7] * U[5]) - U[3] * (U[1] * U[8] - U[7] * U[2]) +
                U[6] * (U[1] * U[5] - U[4] * U[2]);
  double detV = V[0] * (V[4] * V[8] - V[7] * V[5]) - V[3] * (V[1] * V[8] - V[7] * V[2]) +
                V[6] * (V[1] * V[5] - V[4] * V[2]);
  if (detU * detV < 0) {
    // Improper U V^T: flip the singular vector pair with the smallest singular value.
    int cmin = 0;
    for (int c = 1; c < 3; ++c)
      if (nrm[c] < nrm[cmin]) cmin = c;
    for (int r = 0; r < 3; ++r) U[3 * r + cmin] = -U[3 * r + cmin];
  }
  (void)detF;
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) {
      double s = 0;
      for (int c = 0; c < 3; ++c) s += U[3 * a + c] * V[3 * b + c];
      R[3 * a + b] = s;
    }
}

// Float32 polar rotation with the device library's operation order (Newton
// iteration with Frobenius scaling, one-sided Jacobi fallback for det <= 1e-20).
// Selected by polar_mode = 1 so that a parity run isolates the grid-sum order.
inline float det3f(const float* a) {
  float t0 = a[4] * a[8] - a[7] * a[5];
  float t1 = a[1] * a[8] - a[7] * a[2];
  float t2 = a[1] * a[5] - a[4] * a[2];
  float d = a[0] * t0 - a[3] * t1;
  return d + a[6] * t2;
}

inline float dot3f(float a0, float a1, float a2, float b0, float b1, float b2) {
  float s = a0 * b0;
  s = s + a1 * b1;
  return s + a2 * b2;
}

inline void polar_jacobi_f32(const float* F, float* R) {
  float A[9], V[9] = {1.f, 0.f, 0.f, 0.f, 1.f, 0.f, 0.f, 0.f, 1.f};
  for (int i = 0; i < 9; ++i) A[i] = F[i];
  for (int sweep = 0; sweep < 8; ++sweep) {
    float off = 0.f;
    for (int pq = 0; pq < 3; ++pq) {
      const int p = pq == 2 ? 1 : 0, q = pq == 0 ? 1 : 2;
      const float alpha = dot3f(A[p], A[3 + p], A[6 + p], A[p], A[3 + p], A[6 + p]);
      const float beta = dot3f(A[q], A[3 + q], A[6 + q], A[q], A[3 + q], A[6 + q]);
      const float gamma = dot3f(A[p], A[3 + p], A[6 + p], A[q], A[3 + q], A[6 + q]);
      if (gamma == 0.f) continue;
      off = std::fmax(off, std::fabs(gamma) / std::sqrt(alpha * beta));
      const float zeta = (beta - alpha) / (2.f * gamma);
      const float t = std::copysign(1.f, zeta) / (std::fabs(zeta) + std::sqrt(1.f + zeta * zeta));
      const float c = 1.f / std::sqrt(1.f + t * t), s = c * t;
      for (int r = 0; r < 3; ++r) {
        const float ap = A[3 * r + p], aq = A[3 * r + q];
        A[3 * r + p] = c * ap - s * aq;
        A[3 * r + q] = s * ap + c * aq;
        const float vp = V[3 * r + p], vq = V[3 * r + q];
        V[3 * r + p] = c * vp - s * vq;
        V[3 * r + q] = s * vp + c * vq;
      }
    }
    if (off < 1e-7f) break;
  }
  float nrm[3];
  for (int c = 0; c < 3; ++c) nrm[c] = std::sqrt(A[c] * A[c] + A[3 + c] * A[3 + c] + A[6 + c] * A[6 + c]);
  float U[9];
  for (int c = 0; c < 3; ++c)
    for (int r = 0; r < 3; ++r) U[3 * r + c] = nrm[c] > 0.f ? A[3 * r + c] / nrm[c] : (r == c ? 1.f : 0.f);
  if (det3f(U) * det3f(V) < 0.f) {
    int cmin = 0;
    if (nrm[1] < nrm[cmin]) cmin = 1;
    if (nrm[2] < nrm[cmin]) cmin = 2;
    for (int r = 0; r < 3; ++r) U[3 * r + cmin] = -U[3 * r + cmin];
  }
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b)
      R[3 * a + b] = U[3 * a] * V[3 * b] + U[3 * a + 1] * V[3 * b + 1] + U[3 * a + 2] * V[3 * b + 2];
}

inline void polar_newton_f32(const float* F, float* R) {
  float X[9];
  for (int i = 0; i < 9; ++i) X[i] = F[i];
  if (!(det3f(F) > 1e-20f)) {
    polar_jacobi_f32(F, R);
    return;
  }
  bool scale = true;
  for (int it = 0; it < 16; ++it) {
    float Cf[9];
    Cf[0] = X[4] * X[8] - X[5] * X[7];
    Cf[1] = X[5] * X[6] - X[3] * X[8];
    Cf[2] = X[3] * X[7] - X[4] * X[6];
    Cf[3] = X[2] * X[7] - X[1] * X[8];
    Cf[4] = X[0] * X[8] - X[2] * X[6];
    Cf[5] = X[1] * X[6] - X[0] * X[7];
    Cf[6] = X[1] * X[5] - X[2] * X[4];
    Cf[7] = X[2] * X[3] - X[0] * X[5];
    Cf[8] = X[0] * X[4] - X[1] * X[3];
    const float det = X[0] * Cf[0] + X[1] * Cf[1] + X[2] * Cf[2];
    float z = 1.f;
    if (scale) {
      float nx2 = 0.f, nc2 = 0.f;
      for (int i = 0; i < 9; ++i) { nx2 += X[i] * X[i]; nc2 += Cf[i] * Cf[i]; }
      z = std::sqrt(std::sqrt(nc2 / nx2) / std::fabs(det));
    }
    const float a = 0.5f * z, b = 0.5f / (z * det);
    float d2 = 0.f, n2 = 0.f;
    for (int i = 0; i < 9; ++i) {
      const float xn = a * X[i] + b * Cf[i];
      const float dd = xn - X[i];
      d2 += dd * dd;
      n2 += xn * xn;
      X[i] = xn;
    }
    if (d2 < 1e-4f * n2) scale = false;
    if (d2 <= 1e-13f * n2) break;
  }
  for (int i = 0; i < 9; ++i) R[i] = X[i];
}

template <class T>
struct MpmParams {
  T dt, dx, inv_dx, mu, lam, gravity[3], damping;
  int bw, apic;
  int polar_mode;  // 0: exact (float64 Jacobi SVD), 1: device float32 Newton
  int material;    // 0: fixed-corotated (reference), 1: Neo-Hookean extension
};

// Per-particle quantities of one P2G evaluation: the particle's stencil and the terms of
// its grid contributions (mpm3d.py:236-256).
template <class T>
struct P2GPrep {
  int base[3];
  T fx[3];
  T w[3][3];  // w[i][axis]
  T affine[9];
  T mv[3], dtf[3];
  T m;
};

// The part of p2g (mpm3d.py:236-256) that runs once per particle: F <- (I + dt C) F,
// the stress and the affine term. F is written back.
template <class T>
inline void p2g_prepare(int p, const Particles<T>& P, const MpmParams<T>& mp, P2GPrep<T>& r) {
  T x[3] = {P.x[3 * p], P.x[3 * p + 1], P.x[3 * p + 2]};
  base_fx(x, mp.inv_dx, r.base, r.fx);
  for (int a = 0; a < 3; ++a) {
    T ww[3];
    bspline(r.fx[a], ww);
    for (int i = 0; i < 3; ++i) r.w[i][a] = ww[i];
  }
  const T dt = mp.dt;
  T* Cp = P.C + 9 * p;
  T* Fp = P.Fd + 9 * p;
  // F <- (I + dt C) F, mpm3d.py:243.
  T A[9];
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) A[3 * a + b] = (T)(a == b ? 1 : 0) + dt * Cp[3 * a + b];
  T Fn[9];
  matmul3(A, Fp, Fn);
  for (int i = 0; i < 9; ++i) Fp[i] = Fn[i];
  T J = det3(Fn);
  const T mu = P.mu_p ? P.mu_p[p] : mp.mu;
  const T lam = P.lam_p ? P.lam_p[p] : mp.lam;
  T Ft[9];
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) Ft[3 * a + b] = Fn[3 * b + a];
  T stress[9];
  if (mp.material == 1) {
    // Compressible Neo-Hookean Kirchhoff stress mu (F F^T - I) + lam ln(J) I (extension).
    matmul3(Fn, Ft, stress);
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) stress[3 * a + b] = mu * (stress[3 * a + b] - (T)(a == b ? 1 : 0));
    T ll = lam * std::log(J);
    for (int a = 0; a < 3; ++a) stress[4 * a] = stress[4 * a] + ll;
  } else {
    T R[9];
    if (mp.polar_mode == 1 && sizeof(T) == sizeof(float)) {
      float Ff[9], Rf[9];
      for (int i = 0; i < 9; ++i) Ff[i] = (float)Fn[i];
      polar_newton_f32(Ff, Rf);
      for (int i = 0; i < 9; ++i) R[i] = (T)Rf[i];
    } else {
      double Fd64[9], R64[9];
      for (int i = 0; i < 9; ++i) Fd64[i] = (double)Fn[i];
      polar_rotation_f64(Fd64, R64);
      for (int i = 0; i < 9; ++i) R[i] = (T)R64[i];
    }
    // stress = 2 mu (F - R) F^T + lam J (J - 1) I, mpm3d.py:247-251.
    T twomu = (T)2.0 * mu;
    T Pm[9];
    for (int i = 0; i < 9; ++i) Pm[i] = twomu * (Fn[i] - R[i]);
    matmul3(Pm, Ft, stress);
    T lj = (lam * J) * (J - (T)1.0);
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) stress[3 * a + b] = stress[3 * a + b] + lj * (T)(a == b ? 1 : 0);
  }
  T coef = (((-dt) * P.vol[p]) * (T)4.0) * mp.inv_dx;
  coef = coef * mp.inv_dx;
  r.m = P.mass[p];
  for (int i = 0; i < 9; ++i) r.affine[i] = coef * stress[i] + r.m * Cp[i];
  for (int a = 0; a < 3; ++a) {
    r.mv[a] = r.m * P.v[3 * p + a];
    r.dtf[a] = dt * P.fp[3 * p + a];
  }
}

// Contribution of a prepared particle to stencil node (i, j, k) (mpm3d.py:253-266):
// add[0..2] to grid_v, add[3] to grid_m.
template <class T>
inline void p2g_contrib(const P2GPrep<T>& r, int i, int j, int k, T dx, T add[4]) {
  T dpos[3] = {((T)i - r.fx[0]) * dx, ((T)j - r.fx[1]) * dx, ((T)k - r.fx[2]) * dx};
  T weight = (r.w[i][0] * r.w[j][1]) * r.w[k][2];
  for (int a = 0; a < 3; ++a) {
    T ad = r.affine[3 * a] * dpos[0];
    ad = ad + r.affine[3 * a + 1] * dpos[1];
    ad = ad + r.affine[3 * a + 2] * dpos[2];
    T mom = (r.mv[a] + ad) + r.dtf[a];
    add[a] = weight * mom;
  }
  add[3] = weight * r.m;
}

template <class T>
inline void p2g_particle(int p, const Particles<T>& P, Grid<T>& G, const MpmParams<T>& mp,
                         bool atomic) {
  if (P.active[p] == 0) return;
  P2GPrep<T> r;
  p2g_prepare(p, P, mp, r);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      for (int k = 0; k < 3; ++k) {
        int ni = r.base[0] + i, nj = r.base[1] + j, nk = r.base[2] + k;
        if (!G.inside(ni, nj, nk)) continue;
        long c = G.cell(ni, nj, nk);
        T add[4];
        p2g_contrib(r, i, j, k, mp.dx, add);
        for (int a = 0; a < 3; ++a) {
          if (atomic) {
#pragma omp atomic
            G.gv[3 * c + a] += add[a];
          } else {
            G.gv[3 * c + a] = G.gv[3 * c + a] + add[a];
          }
        }
        if (atomic) {
#pragma omp atomic
          G.gm[c] += add[3];
        } else {
          G.gm[c] = G.gm[c] + add[3];
        }
      }
}

// ------------------------------------------------------- cell-ordered sums -
// The summation order of the GPU's sorted, atomic-free scatter. Particles are grouped by
// their base cell b = trunc(x / dx - 0.5); a cell takes part when b lies in [-2, n - 1] on
// every axis (otherwise none of its stencil nodes is in the grid). For each cell and each
// of the 27 stencil offsets o the contributions of its particles are summed sequentially
// in ascending particle index, starting from zero: the cell partial S_b(o). A node's value
// is then its value before the scatter plus the partials S_b(node - b) of its non-empty
// cells b added one at a time in ascending linear cell index, which is descending
// lexicographic o = (2,2,2), (2,2,1), ..., (0,0,0). Each contribution itself is the
// reference's expression, so only the order of the additions differs from a serial loop.
struct CellGroups {
  int ex, ey, ez;                 // extended cell grid [-2, n-1] per axis
  std::vector<int> first, count;  // per group: range in `members`
  std::vector<int> members;       // particle indices, grouped, ascending within a group
  std::vector<int> group_of;      // extended cell -> group id or -1
  long ext(int i, int j, int k) const { return ((long)(i + 2) * ey + (j + 2)) * ez + (k + 2); }
};

// Groups the particles p with include[p] by base cell.
inline void build_cell_groups(int nx, int ny, int nz, int n, const int* base3,
                              const std::vector<char>& include, CellGroups& g) {
  g.ex = nx + 2; g.ey = ny + 2; g.ez = nz + 2;
  const long ncell = (long)g.ex * g.ey * g.ez;
  g.group_of.assign(ncell, -1);
  std::vector<int> cnt;
  for (int p = 0; p < n; ++p) {
    if (!include[p]) continue;
    const int* b = base3 + 3 * p;
    long c = g.ext(b[0], b[1], b[2]);
    if (g.group_of[c] < 0) { g.group_of[c] = (int)cnt.size(); cnt.push_back(0); }
    ++cnt[g.group_of[c]];
  }
  const int ng = (int)cnt.size();
  g.first.assign(ng, 0);
  g.count.assign(ng, 0);
  int run = 0;
  for (int i = 0; i < ng; ++i) { g.first[i] = run; run += cnt[i]; }
  g.members.assign(run, 0);
  for (int p = 0; p < n; ++p) {  // ascending p keeps each group in index order
    if (!include[p]) continue;
    const int* b = base3 + 3 * p;
    int gid = g.group_of[g.ext(b[0], b[1], b[2])];
    g.members[g.first[gid] + g.count[gid]++] = p;
  }
}

inline bool base_in_cell_range(const int b[3], int nx, int ny, int nz) {
  return b[0] >= -2 && b[0] < nx && b[1] >= -2 && b[1] < ny && b[2] >= -2 && b[2] < nz;
}

// p2g in the cell order (all active particles are prepared: F is updated for each).
template <class T>
void p2g_cell_order(const Particles<T>& P, Grid<T>& G, const MpmParams<T>& mp) {
  const int n = P.n;
  std::vector<P2GPrep<T>> prep(n);
  std::vector<int> base3(3 * (size_t)n, 0);
  std::vector<char> include(n, 0);
  for (int p = 0; p < n; ++p) {
    if (P.active[p] == 0) continue;
    p2g_prepare(p, P, mp, prep[p]);
    for (int a = 0; a < 3; ++a) base3[3 * p + a] = prep[p].base[a];
    include[p] = base_in_cell_range(prep[p].base, G.nx, G.ny, G.nz);
  }
  CellGroups g;
  build_cell_groups(G.nx, G.ny, G.nz, n, base3.data(), include, g);
  const int ng = (int)g.first.size();
  std::vector<T> S((size_t)ng * 27 * 4, (T)0);
  for (int gi = 0; gi < ng; ++gi) {
    for (int o = 0; o < 27; ++o) {
      const int i = o / 9, j = (o / 3) % 3, k = o % 3;
      T acc[4] = {0, 0, 0, 0};
      for (int m = 0; m < g.count[gi]; ++m) {
        T add[4];
        p2g_contrib(prep[g.members[g.first[gi] + m]], i, j, k, mp.dx, add);
        for (int a = 0; a < 4; ++a) acc[a] = acc[a] + add[a];
      }
      for (int a = 0; a < 4; ++a) S[((size_t)gi * 27 + o) * 4 + a] = acc[a];
    }
  }
  for (int ni = 0; ni < G.nx; ++ni)
    for (int nj = 0; nj < G.ny; ++nj)
      for (int nk = 0; nk < G.nz; ++nk) {
        const long c = G.cell(ni, nj, nk);
        T acc[4] = {G.gv[3 * c], G.gv[3 * c + 1], G.gv[3 * c + 2], G.gm[c]};
        for (int o = 26; o >= 0; --o) {
          const int i = o / 9, j = (o / 3) % 3, k = o % 3;
          const int gi = g.group_of[g.ext(ni - i, nj - j, nk - k)];
          if (gi < 0) continue;
          for (int a = 0; a < 4; ++a) acc[a] = acc[a] + S[((size_t)gi * 27 + o) * 4 + a];
        }
        G.gv[3 * c] = acc[0]; G.gv[3 * c + 1] = acc[1]; G.gv[3 * c + 2] = acc[2];
        G.gm[c] = acc[3];
      }
}

// grid_op, fsi/mpm3d.py:268-288.
template <class T>
void grid_op(Grid<T>& G, const MpmParams<T>& mp, int nthreads) {
  const T dtg[3] = {mp.dt * mp.gravity[0], mp.dt * mp.gravity[1], mp.dt * mp.gravity[2]};
  const T nd = -mp.damping;
#pragma omp parallel for schedule(static) num_threads(nthreads_or_default(nthreads))
  for (int i = 0; i < G.nx; ++i)
    for (int j = 0; j < G.ny; ++j)
      for (int k = 0; k < G.nz; ++k) {
        long c = G.cell(i, j, k);
        T m = G.gm[c];
        if (!(m > (T)0)) continue;
        T* gv = G.gv + 3 * c;
        for (int a = 0; a < 3; ++a) gv[a] = gv[a] / m;
        for (int a = 0; a < 3; ++a) gv[a] = gv[a] + dtg[a];
        const int node[3] = {i, j, k};
        const int n[3] = {G.nx, G.ny, G.nz};
        for (int a = 0; a < 3; ++a) {
          if (node[a] < mp.bw && gv[a] < (T)0) gv[a] = nd * gv[a];
          if (node[a] >= n[a] - mp.bw && gv[a] > (T)0) gv[a] = nd * gv[a];
        }
      }
}

// g2p + _clamp_particle_position, fsi/mpm3d.py:290-328.
template <class T>
inline void g2p_particle(int p, Particles<T>& P, const Grid<T>& G, const MpmParams<T>& mp,
                         const T lower, const T upper[3]) {
  if (P.active[p] == 0) return;
  T x[3] = {P.x[3 * p], P.x[3 * p + 1], P.x[3 * p + 2]};
  int base[3];
  T fx[3];
  base_fx(x, mp.inv_dx, base, fx);
  T w[3][3];
  for (int a = 0; a < 3; ++a) {
    T ww[3];
    bspline(fx[a], ww);
    for (int i = 0; i < 3; ++i) w[i][a] = ww[i];
  }
  T nv[3] = {0, 0, 0};
  T nc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  const T four_inv_dx = (T)4.0 * mp.inv_dx;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      for (int k = 0; k < 3; ++k) {
        int ni = base[0] + i, nj = base[1] + j, nk = base[2] + k;
        if (!G.inside(ni, nj, nk)) continue;
        T dpos[3] = {(T)i - fx[0], (T)j - fx[1], (T)k - fx[2]};
        T weight = (w[i][0] * w[j][1]) * w[k][2];
        const T* gv = G.gv + 3 * G.cell(ni, nj, nk);
        for (int a = 0; a < 3; ++a) nv[a] = nv[a] + weight * gv[a];
        T s = four_inv_dx * weight;
        for (int a = 0; a < 3; ++a)
          for (int b = 0; b < 3; ++b) nc[3 * a + b] = nc[3 * a + b] + s * (gv[a] * dpos[b]);
      }
  for (int a = 0; a < 3; ++a) P.v[3 * p + a] = nv[a];
  for (int i = 0; i < 9; ++i) P.C[9 * p + i] = mp.apic ? nc[i] : (T)0;
  for (int a = 0; a < 3; ++a) {
    T xa = P.x[3 * p + a] + mp.dt * nv[a];
    xa = std::fmin(std::fmax(xa, lower), upper[a]);
    P.x[3 * p + a] = xa;
  }
}

}  // namespace

// ------------------------------------------------------------ C interface --
// All functions take the reference numpy layouts. `nthreads` <= 0 means 1.

#define FSI_ORACLE_EXPORT extern "C" __attribute__((visibility("default")))

template <class T>
static void lbm_step_impl(int nx, int ny, int nz, T* f, T* F, T* rho, T* v, const T* force,
                          const int32_t* solid, const T* M, const T* invM, const T* S, const T* w,
                          int bc_left, int bc_right, T bc_rho_l, T bc_rho_r, const T* bc_vel_l,
                          const T* bc_vel_r, T rho0, int nthreads) {
  Lattice<T> L{nx, ny, nz, M, invM, S, w};
  collide(L, f, F, rho, v, force, solid, nthreads);
  stream(L, f, F, solid, nthreads);
  apply_boundary_face(L, F, v, solid, 0, 1, bc_left, bc_rho_l, bc_vel_l, rho0);
  apply_boundary_face(L, F, v, solid, nx - 1, nx - 2, bc_right, bc_rho_r, bc_vel_r, rho0);
  update_macro(L, f, F, rho, v, force, solid, rho0, nthreads);
}

// fsi/lbm3d.py:427-433: collide -> stream -> apply_boundary -> update_macro.
FSI_ORACLE_EXPORT void oracle_lbm_step_f32(int nx, int ny, int nz, float* f, float* F, float* rho,
                                           float* v, const float* force, const int32_t* solid,
                                           const float* M, const float* invM, const float* S,
                                           const float* w, int bc_left, int bc_right,
                                           float bc_rho_l, float bc_rho_r, const float* bc_vel_l,
                                           const float* bc_vel_r, float rho0, int nthreads) {
  lbm_step_impl<float>(nx, ny, nz, f, F, rho, v, force, solid, M, invM, S, w, bc_left, bc_right,
                       bc_rho_l, bc_rho_r, bc_vel_l, bc_vel_r, rho0, nthreads);
}

FSI_ORACLE_EXPORT void oracle_lbm_step_f64(int nx, int ny, int nz, double* f, double* F,
                                           double* rho, double* v, const double* force,
                                           const int32_t* solid, const double* M,
                                           const double* invM, const double* S, const double* w,
                                           int bc_left, int bc_right, double bc_rho_l,
                                           double bc_rho_r, const double* bc_vel_l,
                                           const double* bc_vel_r, double rho0, int nthreads) {
  lbm_step_impl<double>(nx, ny, nz, f, F, rho, v, force, solid, M, invM, S, w, bc_left, bc_right,
                        bc_rho_l, bc_rho_r, bc_vel_l, bc_vel_r, rho0, nthreads);
}

// init_fields, fsi/lbm3d.py:256-267.
template <class T>
static void lbm_init_impl(int nx, int ny, int nz, T* f, T* F, T* rho, T* v, const int32_t* solid,
                          const T* w, T rho0, const T* u0) {
  Lattice<T> L{nx, ny, nz, nullptr, nullptr, nullptr, w};
  for (long c = 0; c < L.ncell(); ++c) {
    rho[c] = rho0;
    T u[3] = {u0[0], u0[1], u0[2]};
    if (solid[c] != 0) u[0] = u[1] = u[2] = 0;
    for (int a = 0; a < 3; ++a) v[3 * c + a] = u[a];
    for (int q = 0; q < Q; ++q) {
      T val = feq(L, q, rho[c], u);
      f[c * Q + q] = val;
      F[c * Q + q] = val;
    }
  }
}

FSI_ORACLE_EXPORT void oracle_lbm_init_f32(int nx, int ny, int nz, float* f, float* F, float* rho,
                                           float* v, const int32_t* solid, const float* w,
                                           float rho0, const float* u0) {
  lbm_init_impl<float>(nx, ny, nz, f, F, rho, v, solid, w, rho0, u0);
}

FSI_ORACLE_EXPORT void oracle_lbm_init_f64(int nx, int ny, int nz, double* f, double* F,
                                           double* rho, double* v, const int32_t* solid,
                                           const double* w, double rho0, const double* u0) {
  lbm_init_impl<double>(nx, ny, nz, f, F, rho, v, solid, w, rho0, u0);
}

// MPMSolver3D.substep, fsi/mpm3d.py:189-203: clear_grid -> p2g -> grid_op -> g2p.
// `deterministic` 1 runs P2G serially in particle order, 2 in the cell order above;
// 0 runs it on `nthreads` threads with atomic adds, like a parallel Taichi CPU loop.
template <class T>
static void mpm_substep_impl(int nx, int ny, int nz, int n, T* x, T* v, T* C, T* Fd, const T* mass,
                             const T* vol, const int32_t* active, T* fp, T* gv, T* gm, T dt, T dx,
                             T inv_dx, T mu, T lam, const T* gravity, int bw, T damping, int apic,
                             T lower, const T* upper, int nthreads, int deterministic,
                             int polar_mode, const T* mu_p, const T* lam_p, int material) {
  Particles<T> P{n, x, v, C, Fd, mass, vol, active, fp, mu_p, lam_p};
  Grid<T> G{nx, ny, nz, gv, gm};
  MpmParams<T> mp{dt, dx, inv_dx, mu, lam, {gravity[0], gravity[1], gravity[2]}, damping, bw, apic,
                  polar_mode, material};
  const long N = (long)nx * ny * nz;
  std::memset(gv, 0, sizeof(T) * 3 * N);
  std::memset(gm, 0, sizeof(T) * N);
  if (deterministic == 2) {
    p2g_cell_order(P, G, mp);
  } else if (deterministic) {
    for (int p = 0; p < n; ++p) p2g_particle(p, P, G, mp, false);
  } else {
#pragma omp parallel for schedule(static) num_threads(nthreads_or_default(nthreads))
    for (int p = 0; p < n; ++p) p2g_particle(p, P, G, mp, true);
  }
  grid_op(G, mp, deterministic ? 1 : nthreads);
#pragma omp parallel for schedule(static) num_threads(nthreads_or_default(nthreads))
  for (int p = 0; p < n; ++p) g2p_particle(p, P, G, mp, lower, upper);
}

FSI_ORACLE_EXPORT void oracle_mpm_substep_f32(int nx, int ny, int nz, int n, float* x, float* v,
                                              float* C, float* Fd, const float* mass,
                                              const float* vol, const int32_t* active, float* fp,
                                              float* gv, float* gm, float dt, float dx,
                                              float inv_dx, float mu, float lam,
                                              const float* gravity, int bw, float damping, int apic,
                                              float lower, const float* upper, int nthreads,
                                              int deterministic, int polar_mode,
                                              const float* mu_p, const float* lam_p, int material) {
  mpm_substep_impl<float>(nx, ny, nz, n, x, v, C, Fd, mass, vol, active, fp, gv, gm, dt, dx, inv_dx,
                          mu, lam, gravity, bw, damping, apic, lower, upper, nthreads,
                          deterministic, polar_mode, mu_p, lam_p, material);
}

FSI_ORACLE_EXPORT void oracle_mpm_substep_f64(int nx, int ny, int nz, int n, double* x, double* v,
                                              double* C, double* Fd, const double* mass,
                                              const double* vol, const int32_t* active, double* fp,
                                              double* gv, double* gm, double dt, double dx,
                                              double inv_dx, double mu, double lam,
                                              const double* gravity, int bw, double damping,
                                              int apic, double lower, const double* upper,
                                              int nthreads, int deterministic, int polar_mode,
                                              const double* mu_p, const double* lam_p, int material) {
  mpm_substep_impl<double>(nx, ny, nz, n, x, v, C, Fd, mass, vol, active, fp, gv, gm, dt, dx,
                           inv_dx, mu, lam, gravity, bw, damping, apic, lower, upper, nthreads,
                           deterministic, polar_mode, mu_p, lam_p, material);
}

// Polar rotation of 3x3 float32 matrices with the device operation order.
FSI_ORACLE_EXPORT void oracle_polar_newton_f32(int n, const float* F, float* R) {
  for (int i = 0; i < n; ++i) polar_newton_f32(F + 9 * i, R + 9 * i);
}

// Polar rotation of 3x3 matrices (row-major), for checking the device routine.
FSI_ORACLE_EXPORT void oracle_polar_rotation_f64(int n, const double* F, double* R) {
  for (int i = 0; i < n; ++i) polar_rotation_f64(F + 9 * i, R + 9 * i);
}

// _compute_coupling_forces_kernel, fsi/coupling.py:332-406. With cell_order == 0 the
// reaction and solid fraction are spread in serial particle order; with cell_order != 0 in
// the cell order of p2g_cell_order (per-cell partials over the coupled particles of the
// cell in ascending index, then each fluid node's partials in ascending cell index).
// counters[0..2] += unsupported, partial, clipped.
template <class T>
static void coupling_impl(int nx, int ny, int nz, int n, const T* x, const T* pv, const T* mass,
                          const T* vol, const int32_t* active, T* fp, const T* lbm_v,
                          const int32_t* solid, T* cforce, T* phi, T* valid_out, int32_t* mask_out,
                          int32_t* counters, T inv_dx, T gamma_eff, T dt_ratio, T cell_volume,
                          int build_fraction, T min_valid_weight, int use_rel, T rel_limit,
                          int use_force_limit, T force_limit, int cell_order, int nthreads) {
  Grid<T> G{nx, ny, nz, nullptr, nullptr};
  // Serial particle order unless nthreads > 1 (then a parallel loop with atomic adds, like
  // the reference's parallel Taichi loop; used for timing) or the cell order is asked for.
  const bool parallel = !cell_order && nthreads > 1;
  const T support_tolerance = (T)1.0e-5;
  struct Spread {
    int base[3];
    T w[3][3];
    T valid, pf[3], vol;
  };
  std::vector<Spread> sp(cell_order ? n : 0);
  std::vector<int> base3(cell_order ? 3 * (size_t)n : 0, 0);
  std::vector<char> include(cell_order ? n : 0, 0);
  // The spread of one coupled particle into stencil node (i, j, k): reaction xyz and, when
  // building it, the solid fraction (coupling.py:389-400).
  auto spread_terms = [&](const Spread& r, int i, int j, int k, T out[4]) {
    T weight = (r.w[i][0] * r.w[j][1]) * r.w[k][2];
    T nw = weight / r.valid;
    for (int a = 0; a < 3; ++a) out[a] = (((-nw) * r.pf[a]) * dt_ratio) / cell_volume;
    out[3] = (nw * r.vol) / cell_volume;
  };
#pragma omp parallel for schedule(static) num_threads(nthreads_or_default(nthreads)) if (parallel)
  for (int p = 0; p < n; ++p) {
    if (active[p] == 0) continue;
    T xp[3] = {x[3 * p], x[3 * p + 1], x[3 * p + 2]};
    Spread r;
    T fx[3];
    base_fx(xp, inv_dx, r.base, fx);
    for (int a = 0; a < 3; ++a) {
      T ww[3];
      bspline(fx[a], ww);
      for (int i = 0; i < 3; ++i) r.w[i][a] = ww[i];
    }
    T valid = 0;
    T uf[3] = {0, 0, 0};
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j)
        for (int k = 0; k < 3; ++k) {
          int ni = r.base[0] + i, nj = r.base[1] + j, nk = r.base[2] + k;
          if (!G.inside(ni, nj, nk)) continue;
          long c = G.cell(ni, nj, nk);
          if (solid[c] != 0) continue;
          T weight = (r.w[i][0] * r.w[j][1]) * r.w[k][2];
          valid = valid + weight;
          for (int a = 0; a < 3; ++a) uf[a] = uf[a] + weight * lbm_v[3 * c + a];
        }
    valid_out[p] = valid;
    if (valid > min_valid_weight) {
      if (valid < (T)1.0 - support_tolerance) {
#pragma omp atomic
        counters[1] += 1;
      }
      T dv[3];
      for (int a = 0; a < 3; ++a) {
        uf[a] = uf[a] / valid;
        dv[a] = uf[a] - pv[3 * p + a];
      }
      int clipped = 0;
      if (use_rel) {
        T nrm = std::sqrt(dot3(dv, dv));
        if (nrm > rel_limit && nrm > (T)0) {
          for (int a = 0; a < 3; ++a) dv[a] = (dv[a] / nrm) * rel_limit;
          clipped = 1;
        }
      }
      T pf[3];
      for (int a = 0; a < 3; ++a) pf[a] = (gamma_eff * mass[p]) * dv[a];
      if (use_force_limit) {
        T nrm = std::sqrt(dot3(pf, pf));
        if (nrm > force_limit && nrm > (T)0) {
          for (int a = 0; a < 3; ++a) pf[a] = (pf[a] / nrm) * force_limit;
          clipped = 1;
        }
      }
      for (int a = 0; a < 3; ++a) fp[3 * p + a] = pf[a];
      mask_out[p] = 1;
      if (clipped) {
#pragma omp atomic
        counters[2] += 1;
      }
      r.valid = valid;
      for (int a = 0; a < 3; ++a) r.pf[a] = pf[a];
      r.vol = vol[p];
      if (cell_order) {
        sp[p] = r;
        for (int a = 0; a < 3; ++a) base3[3 * p + a] = r.base[a];
        include[p] = base_in_cell_range(r.base, nx, ny, nz);
        continue;
      }
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
          for (int k = 0; k < 3; ++k) {
            int ni = r.base[0] + i, nj = r.base[1] + j, nk = r.base[2] + k;
            if (!G.inside(ni, nj, nk)) continue;
            long c = G.cell(ni, nj, nk);
            if (solid[c] != 0) continue;
            T add[4];
            spread_terms(r, i, j, k, add);
            if (parallel) {
              for (int a = 0; a < 3; ++a) {
#pragma omp atomic
                cforce[3 * c + a] += add[a];
              }
              if (build_fraction) {
#pragma omp atomic
                phi[c] += add[3];
              }
            } else {
              for (int a = 0; a < 3; ++a) cforce[3 * c + a] = cforce[3 * c + a] + add[a];
              if (build_fraction) phi[c] = phi[c] + add[3];
            }
          }
    } else {
      fp[3 * p] = fp[3 * p + 1] = fp[3 * p + 2] = 0;
      mask_out[p] = 0;
#pragma omp atomic
      counters[0] += 1;
    }
  }
  if (!cell_order) return;
  CellGroups g;
  build_cell_groups(nx, ny, nz, n, base3.data(), include, g);
  const int ng = (int)g.first.size();
  std::vector<T> S((size_t)ng * 27 * 4, (T)0);
  for (int gi = 0; gi < ng; ++gi)
    for (int o = 0; o < 27; ++o) {
      const int i = o / 9, j = (o / 3) % 3, k = o % 3;
      T acc[4] = {0, 0, 0, 0};
      for (int m = 0; m < g.count[gi]; ++m) {
        T add[4];
        spread_terms(sp[g.members[g.first[gi] + m]], i, j, k, add);
        for (int a = 0; a < 4; ++a) acc[a] = acc[a] + add[a];
      }
      for (int a = 0; a < 4; ++a) S[((size_t)gi * 27 + o) * 4 + a] = acc[a];
    }
  for (int ni = 0; ni < nx; ++ni)
    for (int nj = 0; nj < ny; ++nj)
      for (int nk = 0; nk < nz; ++nk) {
        const long c = G.cell(ni, nj, nk);
        if (solid[c] != 0) continue;
        for (int o = 26; o >= 0; --o) {
          const int i = o / 9, j = (o / 3) % 3, k = o % 3;
          const int gi = g.group_of[g.ext(ni - i, nj - j, nk - k)];
          if (gi < 0) continue;
          const T* s4 = &S[((size_t)gi * 27 + o) * 4];
          for (int a = 0; a < 3; ++a) cforce[3 * c + a] = cforce[3 * c + a] + s4[a];
          if (build_fraction) phi[c] = phi[c] + s4[3];
        }
      }
}

FSI_ORACLE_EXPORT void oracle_coupling_f32(int nx, int ny, int nz, int n, const float* x,
                                           const float* pv, const float* mass, const float* vol,
                                           const int32_t* active, float* fp, const float* lbm_v,
                                           const int32_t* solid, float* cforce, float* phi,
                                           float* valid_out, int32_t* mask_out, int32_t* counters,
                                           float inv_dx, float gamma_eff, float dt_ratio,
                                           float cell_volume, int build_fraction,
                                           float min_valid_weight, int use_rel, float rel_limit,
                                           int use_force_limit, float force_limit,
                                           int cell_order, int nthreads) {
  coupling_impl<float>(nx, ny, nz, n, x, pv, mass, vol, active, fp, lbm_v, solid, cforce, phi,
                       valid_out, mask_out, counters, inv_dx, gamma_eff, dt_ratio, cell_volume,
                       build_fraction, min_valid_weight, use_rel, rel_limit, use_force_limit,
                       force_limit, cell_order, nthreads);
}

FSI_ORACLE_EXPORT void oracle_coupling_f64(int nx, int ny, int nz, int n, const double* x,
                                           const double* pv, const double* mass, const double* vol,
                                           const int32_t* active, double* fp, const double* lbm_v,
                                           const int32_t* solid, double* cforce, double* phi,
                                           double* valid_out, int32_t* mask_out, int32_t* counters,
                                           double inv_dx, double gamma_eff, double dt_ratio,
                                           double cell_volume, int build_fraction,
                                           double min_valid_weight, int use_rel, double rel_limit,
                                           int use_force_limit, double force_limit,
                                           int cell_order, int nthreads) {
  coupling_impl<double>(nx, ny, nz, n, x, pv, mass, vol, active, fp, lbm_v, solid, cforce, phi,
                        valid_out, mask_out, counters, inv_dx, gamma_eff, dt_ratio, cell_volume,
                        build_fraction, min_valid_weight, use_rel, rel_limit, use_force_limit,
                        force_limit, cell_order, nthreads);
}

// _compute_immersed_boundary_force_kernel, fsi/coupling.py:421-452 (serial cell order).
// counters[0..1] = active, clipped; total[3] = summed force.
template <class T>
static void ib_impl(long ncell, const T* phi, const T* rho, const T* v, const int32_t* solid,
                    T* ib, int32_t* counters, T* total, int enabled, T drag, T threshold,
                    int use_max, T max_force) {
  counters[0] = counters[1] = 0;
  total[0] = total[1] = total[2] = 0;
  for (long c = 0; c < ncell; ++c) {
    T f[3] = {0, 0, 0};
    if (enabled != 0 && drag > (T)0 && solid[c] == 0) {
      T ph = phi[c];
      if (ph > (T)0 && ph >= threshold) {
        T s = ((-drag) * ph) * rho[c];
        for (int a = 0; a < 3; ++a) f[a] = s * v[3 * c + a];
        T nrm = std::sqrt(dot3(f, f));
        if (use_max != 0 && nrm > max_force && nrm > (T)0) {
          for (int a = 0; a < 3; ++a) f[a] = (f[a] / nrm) * max_force;
          counters[1] += 1;
        }
        counters[0] += 1;
        for (int a = 0; a < 3; ++a) total[a] = total[a] + f[a];
      }
    }
    for (int a = 0; a < 3; ++a) ib[3 * c + a] = f[a];
  }
}

FSI_ORACLE_EXPORT void oracle_ib_f32(long ncell, const float* phi, const float* rho,
                                     const float* v, const int32_t* solid, float* ib,
                                     int32_t* counters, float* total, int enabled, float drag,
                                     float threshold, int use_max, float max_force) {
  ib_impl<float>(ncell, phi, rho, v, solid, ib, counters, total, enabled, drag, threshold, use_max,
                 max_force);
}

FSI_ORACLE_EXPORT void oracle_ib_f64(long ncell, const double* phi, const double* rho,
                                     const double* v, const int32_t* solid, double* ib,
                                     int32_t* counters, double* total, int enabled, double drag,
                                     double threshold, int use_max, double max_force) {
  ib_impl<double>(ncell, phi, rho, v, solid, ib, counters, total, enabled, drag, threshold,
                  use_max, max_force);
}

// _compute_contact_diagnostics_kernel, fsi/coupling.py:463-496.
// counters[0..1] = candidates, damped.
template <class T>
static void contact_impl(int nx, int ny, int nz, int n, const T* x, T* pv, const int32_t* active,
                         const T* phi, const int32_t* solid, int32_t* mask, int32_t* counters,
                         T inv_dx, int enabled, T threshold, T damping) {
  Grid<T> G{nx, ny, nz, nullptr, nullptr};
  counters[0] = counters[1] = 0;
  for (int p = 0; p < n; ++p) {
    mask[p] = 0;
    if (enabled == 0 || active[p] == 0) continue;
    T xp[3] = {x[3 * p], x[3 * p + 1], x[3 * p + 2]};
    int base[3];
    T fx[3];
    base_fx(xp, inv_dx, base, fx);
    T w[3][3];
    for (int a = 0; a < 3; ++a) {
      T ww[3];
      bspline(fx[a], ww);
      for (int i = 0; i < 3; ++i) w[i][a] = ww[i];
    }
    T dyn = 0, stat = 0;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j)
        for (int k = 0; k < 3; ++k) {
          int ni = base[0] + i, nj = base[1] + j, nk = base[2] + k;
          if (!G.inside(ni, nj, nk)) continue;
          long c = G.cell(ni, nj, nk);
          T weight = (w[i][0] * w[j][1]) * w[k][2];
          dyn = dyn + weight * phi[c];
          if (solid[c] != 0) stat = stat + weight;
        }
    if (dyn >= threshold || stat >= threshold) {
      mask[p] = 1;
      counters[0] += 1;
      if (damping > (T)0) {
        T s = (T)1.0 - damping;
        for (int a = 0; a < 3; ++a) pv[3 * p + a] = pv[3 * p + a] * s;
        counters[1] += 1;
      }
    }
  }
}

FSI_ORACLE_EXPORT void oracle_contact_f32(int nx, int ny, int nz, int n, const float* x, float* pv,
                                          const int32_t* active, const float* phi,
                                          const int32_t* solid, int32_t* mask, int32_t* counters,
                                          float inv_dx, int enabled, float threshold,
                                          float damping) {
  contact_impl<float>(nx, ny, nz, n, x, pv, active, phi, solid, mask, counters, inv_dx, enabled,
                      threshold, damping);
}

FSI_ORACLE_EXPORT void oracle_contact_f64(int nx, int ny, int nz, int n, const double* x,
                                          double* pv, const int32_t* active, const double* phi,
                                          const int32_t* solid, int32_t* mask, int32_t* counters,
                                          double inv_dx, int enabled, double threshold,
                                          double damping) {
  contact_impl<double>(nx, ny, nz, n, x, pv, active, phi, solid, mask, counters, inv_dx, enabled,
                       threshold, damping);
}

FSI_ORACLE_EXPORT int oracle_max_threads() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
