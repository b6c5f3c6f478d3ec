// fd2d_oracle.cpp -- CPU oracle for the fd2dmpi forward / adjoint / imaging path.
//
// TEST INFRASTRUCTURE ONLY.  This file checks results and is never the product: only
// tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it.
// The GB300 engine (swit_gb300/csrc) never links or calls it.
//
// It restates, statement by statement and in the same floating-point evaluation
// order (build with -ffp-contract=off so no FMA is formed), the reference's
// 2-D variable-density acoustic staggered-grid solver:
//   fd2dmpi/fdcore.f90:30-198   staggered42_modeling_is  (forward shot)
//   fd2dmpi/fdcore.f90:202-289  staggered42_reco_it      (reverse reconstruction)
//   fd2dmpi/fdcore.f90:293-375  staggered42_back_it      (adjoint step)
//   fd2dmpi/solver.f90:120-289  adjoint_modeling         (imaging, shot sum, -2/c)
//   fd2dmpi/pml.f90:74-101      setup_pml                (damping profile)
//   fd2dmpi/io.f90:231-300      readvelfile / read_densityfile (edge padding)
//   fd2dmpi/io.f90:777-800      free_surface             (flat fs = npml+1)
//   fd2dmpi/math.f90:342-361    min_value_2d_topo        (vmin below fs)
//   fd2dmpi/global.f90:34-35    c1 = 9/8, c2 = -1/24
//   fd2dmpi/mmi_mpi.f90:52-80   get_assigned             (static shot split)
// Indices are kept 1-based (Fortran) internally; arrays are z-fastest.
//
// Deliberate definitions where the reference is undefined:
//   * staggered42_reco_it reads s(it+1), which is s(nt+1) -- past the end of the
//     source array -- at it = nt (fdcore.f90:253).  Here s(nt+1) = 0.
//   * solver.f90:204-206 zeroes dg/dfw/dbk at the start of every shot, so a rank
//     that owns several shots only contributes its last one to the Allreduce.
//     With one rank per shot (the reference examples run mpiproc = ns) the
//     result is the sum over all shots, which is what this oracle computes.
//
// Pinned against the reference's own recorded output: the dot-product test of
// dev/test/02_adjoint_test.ipynb (cells 3, 9): a = <d, d> = 1.25501e+35 and
// a / b = 1.00000 for its homogeneous 401 x 401 model (tests/test_oracle.py).

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

extern "C" {
typedef struct oracle_desc {
  int32_t nx, nz, npml, nt;
  float dx, dt;
  int32_t free_surface;
  int32_t ns, ngmax;
  const int32_t* ng;  // [ns]
  const float* xs;    // [ns]   source x (m)
  const float* zs;    // [ns]   source z (m)
  const float* xg;    // [ns*ngmax] receiver x (m)
  const float* zg;    // [ns*ngmax] receiver z (m)
  int32_t comp;       // recorded component: 0 = p, 1 = vx (u), 2 = vz (w) (dev/solver/fdcore.f90:154-177)
} oracle_desc;
}

namespace {

// Fortran-style 2-D array a(i1, i2), 1-based, first index fastest.
template <class R>
struct F2 {
  std::vector<R> v;
  int n1 = 0, n2 = 0;
  void init(int a, int b) {
    n1 = a;
    n2 = b;
    v.assign((size_t)a * b, R(0));
  }
  R& operator()(int i, int j) { return v[(size_t)(j - 1) * n1 + (i - 1)]; }
  const R& operator()(int i, int j) const { return v[(size_t)(j - 1) * n1 + (i - 1)]; }
  void zero() { std::fill(v.begin(), v.end(), R(0)); }
};

// Strip length per time step, fdcore.f90:52.
inline int strip_len(int nx, int nz) { return nx * 9 + nz * 6; }

// Model, PML and geometry shared by all shots (solver.f90:50-76).
template <class R>
struct Setup {
  int nx, nz, npml, nt, NX, NZ, fs_flag;
  R dx, dt;
  float dx32, dt32;
  F2<R> c, den, damp_g;  // (NZ, NX)
  std::vector<int> fs;   // fs(1..NX), stored at [ix]
  std::vector<R> damp;   // damp(1..npml)
  R c1, c2;

  void build(const oracle_desc& d, const float* vp, const float* rho) {
    nx = d.nx;
    nz = d.nz;
    npml = d.npml;
    nt = d.nt;
    fs_flag = d.free_surface;
    dx32 = d.dx;
    dt32 = d.dt;
    dx = (R)d.dx;
    dt = (R)d.dt;
    NX = nx + 2 * npml;  // pml.f90:29-30
    NZ = nz + 2 * npml;
    // global.f90:34-35
    c1 = R(9.0) / R(8.0);
    c2 = R(-1.0) / R(24.0);
    c.init(NZ, NX);
    den.init(NZ, NX);
    damp_g.init(NZ, NX);
    // io.f90:777-800 flat topography: fs = npml + 1 + int(0/dx).
    fs.assign(NX + 1, npml + 1);
    // io.f90:243-258 and 280-292: interior read, then columns, then rows.
    pad(c, vp);
    pad(den, rho);
    // math.f90:342-361 called as min_value(c(iz1:iz2,ix1:ix2), nz, nx, fs-npml)
    // (solver.f90:73): the j-th column uses fs(j)-npml for j = 1..nx.
    R vmin = R(10000000000.0);
    for (int i = 1; i <= nz; ++i)
      for (int j = 1; j <= nx; ++j)
        if (i > fs[j] - npml)
          if (vmin > c(npml + i, npml + j)) vmin = c(npml + i, npml + j);
    setup_pml(vmin);
  }

  void pad(F2<R>& m, const float* src) {
    for (int ix = 1; ix <= nx; ++ix)
      for (int iz = 1; iz <= nz; ++iz)
        m(npml + iz, npml + ix) = (R)src[(size_t)(ix - 1) * nz + (iz - 1)];
    for (int ix = 1; ix <= npml; ++ix)
      for (int iz = npml + 1; iz <= npml + nz; ++iz) {
        m(iz, ix) = m(iz, npml + 1);
        m(iz, NX - npml + ix) = m(iz, NX - npml);
      }
    for (int iz = 1; iz <= npml; ++iz)
      for (int ix = 1; ix <= NX; ++ix) {
        m(iz, ix) = m(npml + 1, ix);
        m(NZ - npml + iz, ix) = m(NZ - npml, ix);
      }
  }

  // pml.f90:74-101.  log(1000.0) is the correctly rounded value in R.
  void setup_pml(R vmin) {
    damp.assign(npml + 1, R(0));
    R a = (R)(npml - 1) * dx;
    R l1000 = (R)std::log(1000.0);
    R kappa = R(3.0) * vmin * l1000 / (R(2.0) * a);
    for (int ix = 1; ix <= npml; ++ix) {
      R xa = (R)(ix - 1) * dx / a;
      damp[ix] = kappa * xa * xa;
    }
    for (int ix = 1; ix <= npml; ++ix)
      for (int iz = 1; iz <= NZ; ++iz) {
        damp_g(iz, npml - ix + 1) = damp[ix];
        damp_g(iz, NX + ix - npml) = damp[ix];
      }
    for (int iz = 1; iz <= npml; ++iz)
      for (int ix = 1 + (npml - (iz - 1)); ix <= NX - (npml - (iz - 1)); ++ix) {
        damp_g(npml - iz + 1, ix) = damp[iz];
        damp_g(NZ + iz - npml, ix) = damp[iz];
      }
  }

  // Grid indices of a source/receiver coordinate: npml + int(x/dx) + 1 with the
  // division in single precision, exactly as fdcore.f90:70-71, 124-125.
  int gidx(float x) const { return npml + (int)(x / dx32) + 1; }
};

// One shot's forward run: fdcore.f90:30-198.  Strips are stored in the
// reference's boundary(S, nt) layout (S fastest); csg in [ig][it] layout.
template <class R>
void forward_shot(const Setup<R>& S, const oracle_desc& d, int is, const float* s_in, bool store,
                  R* seis, R* boundary, R* p_end, R* u_end, R* w_end, R* dsave = nullptr) {
  const int NX = S.NX, NZ = S.NZ, npml = S.npml, nt = S.nt, nx = S.nx, nz = S.nz;
  const R dt = S.dt, dx = S.dx, c1 = S.c1, c2 = S.c2;
  const int SL = strip_len(nx, nz);
  F2<R> u, w, p;
  u.init(NZ, NX - 1);
  w.init(NZ - 1, NX);
  p.init(NZ, NX);
  const auto& fs = S.fs;
  std::vector<R> s(nt + 2, R(0));
  for (int it = 1; it <= nt; ++it) s[it] = (R)s_in[it - 1];

  int isx = S.gidx(d.xs[is]);
  int isz = S.gidx(d.zs[is]);
  if (isz == fs[isx]) isz = isz + 1;
  const int ng = d.ng[is];
  std::vector<int> gx(ng), gz(ng);
  for (int ig = 0; ig < ng; ++ig) {
    gx[ig] = S.gidx(d.xg[(size_t)is * d.ngmax + ig]);
    gz[ig] = S.gidx(d.zg[(size_t)is * d.ngmax + ig]);
    if (gz[ig] == fs[gx[ig]]) gz[ig] = gz[ig] + 1;
  }

  for (int it = 2; it <= nt; ++it) {
    // p update, fdcore.f90:77-85
    for (int ix = 3; ix <= NX - 2; ++ix)
      for (int iz = fs[ix] + 1; iz <= NZ - 2; ++iz) {
        R alpha = S.den(iz, ix) * S.c(iz, ix) * S.c(iz, ix) * dt / dx;
        R kappa = S.damp_g(iz, ix) * dt;
        // the divergence term D; the exact adjoint reads it back (dsave)
        const R D = c1 * (u(iz, ix) - u(iz, ix - 1) + w(iz, ix) - w(iz - 1, ix)) +
                    c2 * (u(iz, ix + 1) - u(iz, ix - 2) + w(iz + 1, ix) - w(iz - 2, ix));
        p(iz, ix) = (R(1.0) - kappa) * p(iz, ix) - alpha * D;
        if (dsave) dsave[((size_t)(it - 1) * NX + (ix - 1)) * NZ + (iz - 1)] = D;
      }
    // source, fdcore.f90:88-89
    p(isz, isx) = p(isz, isx) + dt * s[it];
    // free surface, fdcore.f90:92-94 (flat fs: p(fs-1,:) = -p(fs+1,:))
    if (S.fs_flag == 1)
      for (int ix = 1; ix <= NX; ++ix) p(fs[ix] - 1, ix) = -p(fs[ix] + 1, ix);
    // u update, fdcore.f90:97-104
    for (int ix = 2; ix <= NX - 2; ++ix)
      for (int iz = fs[ix]; iz <= NZ - 1; ++iz) {
        R alpha = dt / (S.den(iz, ix) * dx);
        R kappa = R(0.5) * (S.damp_g(iz, ix) + S.damp_g(iz, ix + 1)) * dt;
        u(iz, ix) = (R(1.0) - kappa) * u(iz, ix) -
                    alpha * (c1 * (p(iz, ix + 1) - p(iz, ix)) + c2 * (p(iz, ix + 2) - p(iz, ix - 1)));
      }
    // w update, fdcore.f90:106-113
    for (int ix = 2; ix <= NX - 1; ++ix)
      for (int iz = fs[ix]; iz <= NZ - 2; ++iz) {
        R alpha = dt / (S.den(iz, ix) * dx);
        R kappa = R(0.5) * (S.damp_g(iz, ix) + S.damp_g(iz + 1, ix)) * dt;
        w(iz, ix) = (R(1.0) - kappa) * w(iz, ix) -
                    alpha * (c1 * (p(iz + 1, ix) - p(iz, ix)) + c2 * (p(iz + 2, ix) - p(iz - 1, ix)));
      }
    // fdcore.f90:116-120
    if (S.fs_flag == 1)
      for (int ix = 1; ix <= NX; ++ix) w(fs[ix] - 1, ix) = w(fs[ix], ix);
    // fdcore.f90:123-128; vx / vz receivers record u / w (dev/solver/fdcore.f90:154-177)
    for (int ig = 0; ig < ng; ++ig)
      seis[(size_t)ig * nt + (it - 1)] =
          d.comp == 1 ? u(gz[ig], gx[ig]) : (d.comp == 2 ? w(gz[ig], gx[ig]) : p(gz[ig], gx[ig]));
    // fdcore.f90:130-159
    if (store) {
      R* b = boundary + (size_t)(it - 1) * SL;
      int jj = 0;
      for (int j = npml + 1; j <= NX - npml; ++j) {
        b[jj + 0] = p(NZ - npml, j);
        b[jj + 1] = p(NZ - npml - 1, j);
        b[jj + 2] = w(NZ - npml - 1, j);
        jj += 3;
      }
      for (int j = npml + 1; j <= NZ - npml; ++j) {
        b[jj + 0] = p(j, npml + 1);
        b[jj + 1] = p(j, npml + 2);
        b[jj + 2] = u(j, npml + 1);
        b[jj + 3] = p(j, NX - npml);
        b[jj + 4] = p(j, NX - npml - 1);
        b[jj + 5] = u(j, NX - npml - 1);
        jj += 6;
      }
      for (int j = npml + 1; j <= NX - npml; ++j) {
        b[jj + 0] = p(fs[j], j);
        b[jj + 1] = p(fs[j] + 1, j);
        b[jj + 2] = p(fs[j] + 2, j);
        b[jj + 3] = u(fs[j], j);
        b[jj + 4] = u(fs[j] + 1, j);
        b[jj + 5] = w(fs[j], j);
        jj += 6;
      }
    }
  }
  // fdcore.f90:162-166, interior end states in (nz, nx) layout.
  if (store) {
    for (int ix = 1; ix <= nx; ++ix)
      for (int iz = 1; iz <= nz; ++iz) {
        size_t k = (size_t)(ix - 1) * nz + (iz - 1);
        p_end[k] = p(npml + iz, npml + ix);
        u_end[k] = u(npml + iz, npml + ix);
        w_end[k] = w(npml + iz, npml + ix);
      }
  }
}

// One shot's reverse loop: solver.f90:196-253 with the reco step
// (fdcore.f90:202-289), the adjoint step (fdcore.f90:293-375) and the imaging
// condition (solver.f90:237-239).  dg/dfw/dbk are this shot's (nz, nx) sums.
// adj_seis (optional) records p_bk at the receivers after every adjoint step,
// as the dev solver does (dev/solver/fdsolver.f90:205-216).
template <class R>
void adjoint_shot(const Setup<R>& S, const oracle_desc& d, int is, const float* s_in, const float* sadj_in,
                  const R* boundary, const R* p_end0, const R* u_end0, const R* w_end0, R* dg_out,
                  R* dfw_out, R* dbk_out, R* adj_seis) {
  const int NX = S.NX, NZ = S.NZ, npml = S.npml, nt = S.nt, nx = S.nx, nz = S.nz;
  const R dt = S.dt, dx = S.dx, c1 = S.c1, c2 = S.c2;
  const int SL = strip_len(nx, nz);
  const auto& fs = S.fs;
  const int ng = d.ng[is];
  const int ngmax = d.ngmax;

  // Interior slices of c and den (solver.f90:234 passes c(iz1:iz2,ix1:ix2)).
  auto ci = [&](int iz, int ix) -> R { return S.c(npml + iz, npml + ix); };
  auto deni = [&](int iz, int ix) -> R { return S.den(npml + iz, npml + ix); };
  auto fsi = [&](int ix) -> int { return fs[ix + npml] - npml; };  // fs(ix+npml)-npml

  std::vector<R> s(nt + 2, R(0));  // s(nt+1) = 0, see header.
  for (int it = 1; it <= nt; ++it) s[it] = (R)s_in[it - 1];
  F2<R> sadj;
  sadj.init(nt, ngmax);
  for (int ig = 1; ig <= ng; ++ig)
    for (int it = 1; it <= nt; ++it) sadj(it, ig) = (R)sadj_in[(size_t)(ig - 1) * nt + (it - 1)];

  F2<R> pe, ue, we;
  pe.init(nz, nx);
  ue.init(nz, nx);
  we.init(nz, nx);
  for (size_t k = 0; k < (size_t)nz * nx; ++k) {
    pe.v[k] = p_end0[k];
    ue.v[k] = u_end0[k];
    we.v[k] = w_end0[k];
  }
  F2<R> pb, ub, wb, p0;
  pb.init(NZ, NX);
  ub.init(NZ, NX);
  wb.init(NZ, NX);
  p0.init(NZ, NX);
  F2<R> dg, dfw, dbk;
  dg.init(nz, nx);
  dfw.init(nz, nx);
  dbk.init(nz, nx);

  // reco source position (interior indices), fdcore.f90:217-218
  const int risx = (int)(d.xs[is] / S.dx32) + 1;
  const int risz = (int)(d.zs[is] / S.dx32) + 1;
  // adjoint source positions, fdcore.f90:349-359
  std::vector<int> gx(ng), gz(ng), rz(ng);
  for (int ig = 0; ig < ng; ++ig) {
    gx[ig] = S.gidx(d.xg[(size_t)is * ngmax + ig]);
    gz[ig] = S.gidx(d.zg[(size_t)is * ngmax + ig]);
    rz[ig] = (gz[ig] == fs[gx[ig]]) ? gz[ig] + 1 : gz[ig];
  }

  for (int it = nt; it >= 2; --it) {
    p0.v = pb.v;  // solver.f90:232
    const R* b = boundary + (size_t)(it - 2) * SL;  // boundary(:, it-1)

    // ---- staggered42_reco_it ----
    for (int ix = 2; ix <= nx - 2; ++ix)
      for (int iz = fsi(ix) + 1; iz <= nz - 1; ++iz) {
        R alpha = dt / (deni(iz, ix) * dx);
        ue(iz, ix) = ue(iz, ix) + alpha * (c1 * (pe(iz, ix + 1) - pe(iz, ix)) +
                                           c2 * (pe(iz, ix + 2) - pe(iz, ix - 1)));
      }
    for (int ix = 2; ix <= nx - 1; ++ix)
      for (int iz = fsi(ix) + 1; iz <= nz - 2; ++iz) {
        R alpha = dt / (deni(iz, ix) * dx);
        we(iz, ix) = we(iz, ix) + alpha * (c1 * (pe(iz + 1, ix) - pe(iz, ix)) +
                                           c2 * (pe(iz + 2, ix) - pe(iz - 1, ix)));
      }
    {
      int jj = 0;
      for (int j = 1; j <= nx; ++j) {
        we(nz - 1, j) = b[jj + 2];
        jj += 3;
      }
      for (int j = 1; j <= nz; ++j) {
        ue(j, 1) = b[jj + 2];
        ue(j, nx - 1) = b[jj + 5];
        jj += 6;
      }
    }
    if (risx > 2 && risx < nx - 1 && risz > 3 && risz < nz - 1) {
      R beta = dt;
      if (risz > fsi(risx))
        pe(risz, risx) = pe(risz, risx) - beta * s[it + 1];
      else
        pe(fsi(risx) + 1, risx) = pe(fsi(risx) + 1, risx) - beta * s[it + 1];
    }
    for (int ix = 3; ix <= nx - 2; ++ix)
      for (int iz = fsi(ix) + 2; iz <= nz - 2; ++iz) {
        R alpha = deni(iz, ix) * ci(iz, ix) * ci(iz, ix) * dt / dx;
        pe(iz, ix) = pe(iz, ix) + alpha * (c1 * (ue(iz, ix) - ue(iz, ix - 1) + we(iz, ix) - we(iz - 1, ix)) +
                                           c2 * (ue(iz, ix + 1) - ue(iz, ix - 2) + we(iz + 1, ix) - we(iz - 2, ix)));
      }
    {
      int jj = 0;
      for (int j = 1; j <= nx; ++j) {
        pe(nz, j) = b[jj + 0];
        pe(nz - 1, j) = b[jj + 1];
        jj += 3;
      }
      for (int j = 1; j <= nz; ++j) {
        pe(j, 1) = b[jj + 0];
        pe(j, 2) = b[jj + 1];
        pe(j, nx) = b[jj + 3];
        pe(j, nx - 1) = b[jj + 4];
        jj += 6;
      }
      for (int j = 1; j <= nx; ++j) {
        pe(fsi(j), j) = b[jj + 0];
        pe(fsi(j) + 1, j) = b[jj + 1];
        pe(fsi(j) + 2, j) = b[jj + 2];
        jj += 6;
      }
    }

    // ---- staggered42_back_it ----
    for (int ix = 2; ix <= NX - 2; ++ix)
      for (int iz = 2; iz <= NZ - 1; ++iz) {
        R alpha = S.den(iz, ix) * S.c(iz, ix) * S.c(iz, ix) * dt / dx;
        R kappa = R(0.5) * (S.damp_g(iz, ix) + S.damp_g(iz, ix + 1)) * dt;
        ub(iz, ix) = (R(1.0) - kappa) * ub(iz, ix) -
                     alpha * (c1 * (pb(iz, ix + 1) - pb(iz, ix)) + c2 * (pb(iz, ix + 2) - pb(iz, ix - 1)));
      }
    for (int ix = 2; ix <= NX - 1; ++ix)
      for (int iz = 2; iz <= NZ - 2; ++iz) {
        R alpha = S.den(iz, ix) * S.c(iz, ix) * S.c(iz, ix) * dt / dx;
        R kappa = R(0.5) * (S.damp_g(iz, ix) + S.damp_g(iz + 1, ix)) * dt;
        wb(iz, ix) = (R(1.0) - kappa) * wb(iz, ix) -
                     alpha * (c1 * (pb(iz + 1, ix) - pb(iz, ix)) + c2 * (pb(iz + 2, ix) - pb(iz - 1, ix)));
      }
    if (S.fs_flag == 1)
      for (int ix = 2; ix <= NX - 1; ++ix) wb(fs[ix] - 1, ix) = wb(fs[ix], ix);
    for (int ix = 3; ix <= NX - 2; ++ix)
      for (int iz = 3; iz <= NZ - 2; ++iz) {
        R alpha = dt / (S.den(iz, ix) * dx);
        R kappa = S.damp_g(iz, ix) * dt;
        pb(iz, ix) = (R(1.0) - kappa) * pb(iz, ix) -
                     alpha * (c1 * (ub(iz, ix) - ub(iz, ix - 1) + wb(iz, ix) - wb(iz - 1, ix)) +
                              c2 * (ub(iz, ix + 1) - ub(iz, ix - 2) + wb(iz + 1, ix) - wb(iz - 2, ix)));
      }
    for (int ig = 1; ig <= ng; ++ig) {
      R beta = dt;
      int igx = gx[ig - 1], igz = gz[ig - 1];
      const int z = igz > fs[igx] ? igz : fs[igx] + 1;
      if (d.comp == 1)  // dev/solver/fdcore.f90:472-478
        ub(z, igx) = ub(z, igx) - beta * sadj(it, ig);
      else if (d.comp == 2)  // dev/solver/fdcore.f90:479-485
        wb(z, igx) = wb(z, igx) - beta * sadj(it, ig);
      else
        pb(z, igx) = pb(z, igx) + beta * sadj(it, ig);
    }
    for (int ix = 1; ix <= NX; ++ix) pb(fs[ix] - 1, ix) = -pb(fs[ix] + 1, ix);

    if (adj_seis)
      for (int ig = 0; ig < ng; ++ig) adj_seis[(size_t)ig * nt + (it - 1)] = pb(rz[ig], gx[ig]);

    // ---- imaging, solver.f90:237-239 ----
    for (int ix = 1; ix <= nx; ++ix)
      for (int iz = 1; iz <= nz; ++iz) {
        R pf = pe(iz, ix);
        R pbo = p0(npml + iz, npml + ix);
        R pbn = pb(npml + iz, npml + ix);
        dg(iz, ix) = dg(iz, ix) + pf * (pbo - pbn);
        dfw(iz, ix) = dfw(iz, ix) + pf * pf;
        dbk(iz, ix) = dbk(iz, ix) + pbn * pbn;
      }
  }
  std::memcpy(dg_out, dg.v.data(), sizeof(R) * nz * nx);
  std::memcpy(dfw_out, dfw.v.data(), sizeof(R) * nz * nx);
  std::memcpy(dbk_out, dbk.v.data(), sizeof(R) * nz * nx);
}

// mmi_mpi.f90:52-80, static contiguous split of shots [is1, is2] over nsize ranks.
void get_assigned(int is1, int is2, int rank, int nsize, int& b, int& e) {
  if (nsize == 1) {
    b = is1;
    e = is2;
    return;
  }
  int nnn = is2 - is1 + 1;
  int ii1 = nnn / nsize;
  if (ii1 == 0) {
    b = is1 + rank;
    e = b;
    return;
  }
  int ii2 = nnn - ii1 * nsize;
  if (rank < nsize - ii2) {
    b = is1 + rank * ii1;
    e = is1 + (rank + 1) * ii1 - 1;
  } else {
    b = is1 + ii2 + rank * ii1 + rank - nsize;
    e = is1 + ii2 + (rank + 1) * ii1 + rank - nsize;
  }
}

template <class F>
void run_ranks(int ns, int nthreads, F&& f) {
  if (nthreads < 1) nthreads = 1;
  if (nthreads > ns) nthreads = ns;
  std::vector<std::thread> th;
  for (int r = 0; r < nthreads; ++r) {
    int b, e;
    get_assigned(1, ns, r, nthreads, b, e);
    if (b > ns) continue;
    if (e > ns) e = ns;
    th.emplace_back([&, b, e]() {
      for (int is = b; is <= e; ++is) f(is - 1);
    });
  }
  for (auto& t : th) t.join();
}

int check_desc(const oracle_desc* d) {
  if (!d) return -1;
  if (d->nx < 8 || d->nz < 8 || d->npml < 2 || d->nt < 2 || d->ns < 1 || d->ngmax < 1) return -2;
  if (d->comp < 0 || d->comp > 2) return -2;
  if (!(d->dx > 0.f) || !(d->dt > 0.f)) return -2;
  const int NX = d->nx + 2 * d->npml, NZ = d->nz + 2 * d->npml;
  auto gi = [&](float x) { return d->npml + (int)(x / d->dx) + 1; };
  for (int is = 0; is < d->ns; ++is) {
    if (d->ng[is] < 0 || d->ng[is] > d->ngmax) return -3;
    int sx = gi(d->xs[is]), sz = gi(d->zs[is]);
    if (sx < 3 || sx > NX - 2 || sz < 3 || sz > NZ - 2) return -4;
    for (int ig = 0; ig < d->ng[is]; ++ig) {
      int gx = gi(d->xg[(size_t)is * d->ngmax + ig]), gz = gi(d->zg[(size_t)is * d->ngmax + ig]);
      if (gx < 3 || gx > NX - 2 || gz < 3 || gz > NZ - 2) return -4;
    }
  }
  return 0;
}

template <class R>
int forward_all(const oracle_desc* d, const float* vp, const float* rho, const float* src, int store, R* seis,
                R* boundary, R* p_end, R* u_end, R* w_end, int nthreads) {
  int rc = check_desc(d);
  if (rc) return rc;
  Setup<R> S;
  S.build(*d, vp, rho);
  const size_t SL = strip_len(d->nx, d->nz), NI = (size_t)d->nx * d->nz;
  std::fill(seis, seis + (size_t)d->ns * d->ngmax * d->nt, R(0));
  if (store) std::fill(boundary, boundary + (size_t)d->ns * d->nt * SL, R(0));
  run_ranks(d->ns, nthreads, [&](int is) {
    forward_shot<R>(S, *d, is, src + (size_t)is * d->nt, store != 0, seis + (size_t)is * d->ngmax * d->nt,
                    store ? boundary + (size_t)is * d->nt * SL : nullptr, store ? p_end + is * NI : nullptr,
                    store ? u_end + is * NI : nullptr, store ? w_end + is * NI : nullptr);
  });
  return 0;
}

// Shot sum in shot order, then g = -2 g / c over the interior (solver.f90:263-270).
template <class R>
void reduce_shots(const Setup<R>& S, int ns, const std::vector<R>& dg, const std::vector<R>& dfw,
                  const std::vector<R>& dbk, R* g, R* fw, R* bk) {
  const size_t NI = (size_t)S.nx * S.nz;
  for (size_t k = 0; k < NI; ++k) {
    R a = dg[k], b = dfw[k], c = dbk[k];
    for (int is = 1; is < ns; ++is) {
      a = a + dg[is * NI + k];
      b = b + dfw[is * NI + k];
      c = c + dbk[is * NI + k];
    }
    int ix = (int)(k / S.nz) + 1, iz = (int)(k % S.nz) + 1;
    g[k] = R(-2.0) * a / S.c(S.npml + iz, S.npml + ix);
    fw[k] = b;
    bk[k] = c;
  }
}

template <class R>
int adjoint_all(const oracle_desc* d, const float* vp, const float* rho, const float* src, const float* adj,
                const R* boundary, const R* p_end, const R* u_end, const R* w_end, R* g, R* fw, R* bk,
                R* adj_seis, int nthreads) {
  int rc = check_desc(d);
  if (rc) return rc;
  Setup<R> S;
  S.build(*d, vp, rho);
  const size_t SL = strip_len(d->nx, d->nz), NI = (size_t)d->nx * d->nz;
  std::vector<R> dg(d->ns * NI), dfw(d->ns * NI), dbk(d->ns * NI);
  if (adj_seis) std::fill(adj_seis, adj_seis + (size_t)d->ns * d->ngmax * d->nt, R(0));
  run_ranks(d->ns, nthreads, [&](int is) {
    adjoint_shot<R>(S, *d, is, src + (size_t)is * d->nt, adj + (size_t)is * d->ngmax * d->nt,
                    boundary + (size_t)is * d->nt * SL, p_end + is * NI, u_end + is * NI, w_end + is * NI,
                    dg.data() + is * NI, dfw.data() + is * NI, dbk.data() + is * NI,
                    adj_seis ? adj_seis + (size_t)is * d->ngmax * d->nt : nullptr);
  });
  reduce_shots(S, d->ns, dg, dfw, dbk, g, fw, bk);
  return 0;
}

// Full shot-gradient for the Waveform (L2) misfit: forward with strips, the
// reference adjoint source syn - obs per live trace (toolbox/misfit.py:128-148),
// then the reverse loop.  Strips live per shot in memory instead of on disk.
template <class R>
int gradient_all(const oracle_desc* d, const float* vp, const float* rho, const float* src, const float* obs, R* g,
                 R* fw, R* bk, R* seis_out, int nthreads) {
  int rc = check_desc(d);
  if (rc) return rc;
  Setup<R> S;
  S.build(*d, vp, rho);
  const size_t SL = strip_len(d->nx, d->nz), NI = (size_t)d->nx * d->nz;
  const size_t NS = (size_t)d->ngmax * d->nt;
  std::vector<R> dg(d->ns * NI), dfw(d->ns * NI), dbk(d->ns * NI);
  run_ranks(d->ns, nthreads, [&](int is) {
    std::vector<R> seis(NS, R(0)), bnd((size_t)d->nt * SL, R(0)), pe(NI), ue(NI), we(NI);
    forward_shot<R>(S, *d, is, src + (size_t)is * d->nt, true, seis.data(), bnd.data(), pe.data(), ue.data(),
                    we.data());
    std::vector<float> adj(NS, 0.f);
    const float* o = obs + (size_t)is * NS;
    for (int ig = 0; ig < d->ng[is]; ++ig) {
      double on = 0, sn = 0;
      for (int it = 0; it < d->nt; ++it) {
        on += (double)o[(size_t)ig * d->nt + it] * o[(size_t)ig * d->nt + it];
        sn += (double)seis[(size_t)ig * d->nt + it] * seis[(size_t)ig * d->nt + it];
      }
      if (on > 0 && sn > 0)
        for (int it = 0; it < d->nt; ++it)
          adj[(size_t)ig * d->nt + it] = (float)((double)(float)seis[(size_t)ig * d->nt + it] -
                                                 (double)o[(size_t)ig * d->nt + it]);
    }
    if (seis_out)
      for (size_t k = 0; k < NS; ++k) seis_out[is * NS + k] = seis[k];
    adjoint_shot<R>(S, *d, is, src + (size_t)is * d->nt, adj.data(), bnd.data(), pe.data(), ue.data(), we.data(),
                    dg.data() + is * NI, dfw.data() + is * NI, dbk.data() + is * NI, nullptr);
  });
  reduce_shots(S, d->ns, dg, dfw, dbk, g, fw, bk);
  return 0;
}

// ---------------------------------------------------------------------------
// Exact discrete adjoint of forward_shot (not a reference algorithm: the
// transpose of the reference's FP forward recursion, fdcore.f90:75-128, for the
// vp gradient and the source gradient).  With the damping held fixed (vmin and
// so the damping profile are treated as constants), step it maps (p, u, w) by
//   S1  p := (1-kp) p - A D(u, w)       on ix in [3,NX-2], iz in [fs+1,NZ-2]
//   S2  p(isz,isx) += dt s(it)
//   S3  p(fs-1,:) := -p(fs+1,:)         (free surface)
//   S4  u := (1-ku) u - B Gx(p)         on ix in [2,NX-2], iz in [fs,NZ-1]
//       w := (1-kw) w - B Gz(p)         on ix in [2,NX-1], iz in [fs,NZ-2]
//   S5  w(fs-1,:) := w(fs,:)            (free surface)
//   S6  seis(ig, it) = p(gz, gx)   (u or w for vx / vz receivers)
// with A = den c^2 dt/dx, B = dt/(den dx).  The adjoint runs it = nt..2 in two
// gather passes per step (the form the GB300 kernels take, so both evaluate the
// same expressions in the same order):
//   K1 (pressure points of S1's range): lp = (1-kp) lp [S1 scaling of step it+1]
//      + adjoint sources [S6] + the S4 transposes from lu, lw~ [w~(fs) = w(fs) +
//      m, the S5 fold] - c2 B(fs) w~(fs) at row fs+1 [S3 fold]; the source
//      gradient dt lp [S2]; gA -= lp D_it [S1]; p := lp (unscaled).
//   K2 (velocity points): lu = (1-ku) lu + S1 transposes from lp; likewise lw
//      from lw~; m_new(ix) = c2 A(fs+1,ix) lp(fs+1,ix) [S1's read of w(fs-1)].
// m alternates between two rows by step parity.  gA is the gradient with respect
// to A per PML point; dJ/dc = gA 2 den c dt/dx, and dJ/dvp sums dJ/dc over the
// PML points padded from each interior point (io.f90:243-292: clamp to the
// interior).  dsave holds D of every step: [it-1][ix-1][iz-1].
template <class R>
void exact_adjoint_shot(const Setup<R>& S, const oracle_desc& d, int is, const float* sadj_in, const R* dsave,
                        R* gA, R* gsrc) {
  const int NX = S.NX, NZ = S.NZ, nt = S.nt;
  const R dt = S.dt, dx = S.dx, c1 = S.c1, c2 = S.c2;
  const auto& fs = S.fs;
  const int F = fs[1];  // flat free surface
  const bool fold = S.fs_flag == 1;
  F2<R> A, B, kp, ku, kw, lp, lu, lw;
  for (F2<R>* a : {&A, &B, &kp, &ku, &kw, &lp, &lu, &lw}) a->init(NZ, NX);
  for (int ix = 1; ix <= NX; ++ix)
    for (int iz = 1; iz <= NZ; ++iz) {
      A(iz, ix) = S.den(iz, ix) * S.c(iz, ix) * S.c(iz, ix) * dt / dx;
      B(iz, ix) = dt / (S.den(iz, ix) * dx);
      kp(iz, ix) = S.damp_g(iz, ix) * dt;
      if (ix + 1 <= NX) ku(iz, ix) = R(0.5) * (S.damp_g(iz, ix) + S.damp_g(iz, ix + 1)) * dt;
      if (iz + 1 <= NZ) kw(iz, ix) = R(0.5) * (S.damp_g(iz, ix) + S.damp_g(iz + 1, ix)) * dt;
    }
  std::vector<R> m[2] = {std::vector<R>(NX + 1, R(0)), std::vector<R>(NX + 1, R(0))};
  int isx = S.gidx(d.xs[is]);
  int isz = S.gidx(d.zs[is]);
  if (isz == fs[isx]) isz = isz + 1;
  const int ng = d.ng[is];
  std::vector<int> gx(ng), gz(ng);
  for (int ig = 0; ig < ng; ++ig) {
    gx[ig] = S.gidx(d.xg[(size_t)is * d.ngmax + ig]);
    gz[ig] = S.gidx(d.zg[(size_t)is * d.ngmax + ig]);
    if (gz[ig] == fs[gx[ig]]) gz[ig] = gz[ig] + 1;
  }
  auto inRp = [&](int iz, int ix) { return ix >= 3 && ix <= NX - 2 && iz >= F + 1 && iz <= NZ - 2; };
  for (int it = 1; it <= nt; ++it) gsrc[it - 1] = R(0);
  for (int it = nt; it >= 2; --it) {
    const std::vector<R>& mo = m[it & 1];
    std::vector<R>& mn = m[(it - 1) & 1];
    auto wt = [&](int iz, int ix) -> R { return (fold && iz == F) ? lw(iz, ix) + mo[ix] : lw(iz, ix); };
    const R* D = dsave + (size_t)(it - 1) * NX * NZ;
    // vx / vz receivers (S6 records u or w): their adjoint sources go into lu or
    // lw before the step's gathers, in receiver order
    if (d.comp != 0)
      for (int ig = 0; ig < ng; ++ig) {
        F2<R>& lr = d.comp == 1 ? lu : lw;
        lr(gz[ig], gx[ig]) = lr(gz[ig], gx[ig]) + (R)sadj_in[(size_t)ig * nt + (it - 1)];
      }
    // K1
    for (int ix = 3; ix <= NX - 2; ++ix)
      for (int iz = F + 1; iz <= NZ - 2; ++iz) {
        R l = (R(1.0) - kp(iz, ix)) * lp(iz, ix);
        if (d.comp == 0)
          for (int ig = 0; ig < ng; ++ig)
            if (gz[ig] == iz && gx[ig] == ix) l = l + (R)sadj_in[(size_t)ig * nt + (it - 1)];
        l = l - c1 * (B(iz, ix - 1) * lu(iz, ix - 1));
        l = l + c1 * (B(iz, ix) * lu(iz, ix));
        if (ix - 2 >= 2) l = l - c2 * (B(iz, ix - 2) * lu(iz, ix - 2));
        if (ix + 1 <= NX - 2) l = l + c2 * (B(iz, ix + 1) * lu(iz, ix + 1));
        l = l - c1 * (B(iz - 1, ix) * wt(iz - 1, ix));
        l = l + c1 * (B(iz, ix) * wt(iz, ix));
        if (iz - 2 >= F) l = l - c2 * (B(iz - 2, ix) * wt(iz - 2, ix));
        if (iz + 1 <= NZ - 2) l = l + c2 * (B(iz + 1, ix) * wt(iz + 1, ix));
        if (fold && iz == F + 1) l = l - c2 * (B(F, ix) * wt(F, ix));
        if (iz == isz && ix == isx) gsrc[it - 1] = dt * l;
        const size_t k = (size_t)(ix - 1) * NZ + (iz - 1);
        gA[k] = gA[k] - l * D[k];
        lp(iz, ix) = l;
      }
    // K2 (reads lp from K1, m[it&1]; writes lu, lw, m[(it-1)&1])
    for (int ix = 2; ix <= NX - 1; ++ix)
      for (int iz = F; iz <= NZ - 1; ++iz) {
        if (ix <= NX - 2) {
          R l = (R(1.0) - ku(iz, ix)) * lu(iz, ix);
          if (inRp(iz, ix)) l = l - c1 * (A(iz, ix) * lp(iz, ix));
          if (inRp(iz, ix + 1)) l = l + c1 * (A(iz, ix + 1) * lp(iz, ix + 1));
          if (inRp(iz, ix - 1)) l = l - c2 * (A(iz, ix - 1) * lp(iz, ix - 1));
          if (inRp(iz, ix + 2)) l = l + c2 * (A(iz, ix + 2) * lp(iz, ix + 2));
          lu(iz, ix) = l;
        }
        if (iz <= NZ - 2) {
          R l = (R(1.0) - kw(iz, ix)) * wt(iz, ix);
          if (inRp(iz, ix)) l = l - c1 * (A(iz, ix) * lp(iz, ix));
          if (inRp(iz + 1, ix)) l = l + c1 * (A(iz + 1, ix) * lp(iz + 1, ix));
          if (inRp(iz - 1, ix)) l = l - c2 * (A(iz - 1, ix) * lp(iz - 1, ix));
          if (inRp(iz + 2, ix)) l = l + c2 * (A(iz + 2, ix) * lp(iz + 2, ix));
          if (fold && iz == F && inRp(F + 1, ix)) mn[ix] = c2 * (A(F + 1, ix) * lp(F + 1, ix));
          lw(iz, ix) = l;
        }
      }
  }
}

// dJ/dvp on the interior (nx, nz) from the per-shot gA sums: shots summed in
// order per PML point, times dA/dc = 2 den c dt/dx, then summed over the PML
// points each interior point was padded to (columns, then rows ascending).
template <class R>
void exact_reduce(const Setup<R>& S, int ns, const std::vector<R>& gA, R* g) {
  const int NX = S.NX, NZ = S.NZ, L = S.npml, nx = S.nx, nz = S.nz;
  const size_t N = (size_t)NX * NZ;
  for (int j = 1; j <= nx; ++j)
    for (int i = 1; i <= nz; ++i) {
      const int x0 = j == 1 ? 1 : L + j, x1 = j == nx ? NX : L + j;
      const int z0 = i == 1 ? 1 : L + i, z1 = i == nz ? NZ : L + i;
      R acc = R(0);
      for (int ix = x0; ix <= x1; ++ix)
        for (int iz = z0; iz <= z1; ++iz) {
          const size_t k = (size_t)(ix - 1) * NZ + (iz - 1);
          R t = gA[k];
          for (int is = 1; is < ns; ++is) t = t + gA[is * N + k];
          const R dadc = R(2.0) * S.den(iz, ix) * S.c(iz, ix) * S.dt / S.dx;
          acc = acc + t * dadc;
        }
      g[(size_t)(j - 1) * nz + (i - 1)] = acc;
    }
}

// Forward of every shot (seismograms, D of every step) and the exact adjoint of
// adjoint sources adj (ns, ngmax, nt): g = dJ/dvp (nx, nz), gsrc = dJ/dsrc (ns, nt).
template <class R>
int exact_all(const oracle_desc* d, const float* vp, const float* rho, const float* src, const float* adj, R* g,
              R* gsrc, R* seis_out, int nthreads) {
  int rc = check_desc(d);
  if (rc) return rc;
  Setup<R> S;
  S.build(*d, vp, rho);
  const size_t N = (size_t)S.NX * S.NZ, NS = (size_t)d->ngmax * d->nt;
  std::vector<R> gA(d->ns * N, R(0));
  run_ranks(d->ns, nthreads, [&](int is) {
    std::vector<R> seis(NS, R(0)), D((size_t)d->nt * N, R(0));
    forward_shot<R>(S, *d, is, src + (size_t)is * d->nt, false, seis.data(), nullptr, nullptr, nullptr, nullptr,
                    D.data());
    if (seis_out)
      for (size_t k = 0; k < NS; ++k) seis_out[is * NS + k] = seis[k];
    exact_adjoint_shot<R>(S, *d, is, adj + (size_t)is * NS, D.data(), gA.data() + is * N,
                          gsrc + (size_t)is * d->nt);
  });
  exact_reduce(S, d->ns, gA, g);
  return 0;
}

}  // namespace

extern "C" {

int oracle_strip_len(int nx, int nz) { return strip_len(nx, nz); }

// Damping profile damp_global(NZ, NX) in float, pml.f90:74-101 (with vmin from
// math.f90:342-361), written z-fastest [NX][NZ].  Used to check the engine's
// closed-form profile.
int oracle_damp_profile_f32(const oracle_desc* d, const float* vp, const float* rho, float* out) {
  if (!d || d->nx < 1 || d->nz < 1 || d->npml < 2) return -2;
  Setup<float> S;
  S.build(*d, vp, rho);
  std::memcpy(out, S.damp_g.v.data(), sizeof(float) * S.damp_g.v.size());
  return 0;
}

int oracle_forward_f32(const oracle_desc* d, const float* vp, const float* rho, const float* src, int store,
                       float* seis, float* boundary, float* p_end, float* u_end, float* w_end, int nthreads) {
  return forward_all<float>(d, vp, rho, src, store, seis, boundary, p_end, u_end, w_end, nthreads);
}
int oracle_forward_f64(const oracle_desc* d, const float* vp, const float* rho, const float* src, int store,
                       double* seis, double* boundary, double* p_end, double* u_end, double* w_end, int nthreads) {
  return forward_all<double>(d, vp, rho, src, store, seis, boundary, p_end, u_end, w_end, nthreads);
}
int oracle_adjoint_f32(const oracle_desc* d, const float* vp, const float* rho, const float* src, const float* adj,
                       const float* boundary, const float* p_end, const float* u_end, const float* w_end, float* g,
                       float* fw, float* bk, float* adj_seis, int nthreads) {
  return adjoint_all<float>(d, vp, rho, src, adj, boundary, p_end, u_end, w_end, g, fw, bk, adj_seis, nthreads);
}
int oracle_adjoint_f64(const oracle_desc* d, const float* vp, const float* rho, const float* src, const float* adj,
                       const double* boundary, const double* p_end, const double* u_end, const double* w_end,
                       double* g, double* fw, double* bk, double* adj_seis, int nthreads) {
  return adjoint_all<double>(d, vp, rho, src, adj, boundary, p_end, u_end, w_end, g, fw, bk, adj_seis, nthreads);
}
int oracle_gradient_f32(const oracle_desc* d, const float* vp, const float* rho, const float* src, const float* obs,
                        float* g, float* fw, float* bk, float* seis, int nthreads) {
  return gradient_all<float>(d, vp, rho, src, obs, g, fw, bk, seis, nthreads);
}
int oracle_gradient_f64(const oracle_desc* d, const float* vp, const float* rho, const float* src, const float* obs,
                        double* g, double* fw, double* bk, double* seis, int nthreads) {
  return gradient_all<double>(d, vp, rho, src, obs, g, fw, bk, seis, nthreads);
}

int oracle_exact_f32(const oracle_desc* d, const float* vp, const float* rho, const float* src, const float* adj,
                     float* g, float* gsrc, float* seis, int nthreads) {
  return exact_all<float>(d, vp, rho, src, adj, g, gsrc, seis, nthreads);
}
int oracle_exact_f64(const oracle_desc* d, const float* vp, const float* rho, const float* src, const float* adj,
                     double* g, double* gsrc, double* seis, int nthreads) {
  return exact_all<double>(d, vp, rho, src, adj, g, gsrc, seis, nthreads);
}

}  // extern "C"
