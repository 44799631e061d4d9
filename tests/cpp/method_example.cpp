// A C++ host using the GB300 VL+CT step through include/mhdvlct_method.hpp,
// the way a Cello glue class would: construct the Method from the
// Method:mhd_vlct parameter text, check the reference's validation errors,
// and (with a GPU) advance one block and compare with a second Method run
// through the plain C ABI.
//
// Usage: method_example              (no GPU needed: construction and errors)
//        method_example --gpu        (also one timestep + compute on cuda:0)
//        method_example --smr FILE   (a two-level mesh on cuda:0: refresh,
//                                     step with stored fluxes, flux correction;
//                                     FILE lists the leaves and refresh faces)
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "mhdvlct_method.hpp"

static const char* kParams =
    "Method { mhd_vlct { mhd_choice = \"constrained_transport\";"
    " riemann_solver = \"hlld\"; reconstruct_method = \"plm\"; courant = 0.4; }; }"
    " Physics { fluid_props { eos { gamma = 1.6666666666666667; }"
    " floors { density = 1e-200; pressure = 1e-200; } } }";

static int fail(const char* what) {
  std::fprintf(stderr, "FAIL: %s\n", what);
  return 1;
}

static const char* kHydroParams =
    "Method { mhd_vlct { mhd_choice = \"no_bfield\"; riemann_solver = \"hllc\";"
    " reconstruct_method = \"plm\"; courant = 0.4; }; }"
    " Physics { fluid_props { eos { gamma = 1.6666666666666667; }"
    " floors { density = 1e-200; pressure = 1e-200; } } }";

// Static mesh refinement through the C++ Method: hydro leaves of n^3 cells
// (ghost depth g) read from `path` (a header "nleaf n g root", one line
// "level ox oy oz" per leaf with its origin in finest cells, then "nfaces"
// and one line of 9 ints per refresh face), a moving density contact, two
// cycles of Cello's order with flux correction; prints the relative change
// of the mass and total-energy totals.
static int run_smr(const char* path) {
  std::ifstream in(path);
  int nleaf = 0, n = 0, g = 0, root = 0;
  if (!(in >> nleaf >> n >> g >> root)) return fail("smr header");
  std::vector<int> level(nleaf), org(3 * (size_t)nleaf);
  int max_level = 0;
  for (int i = 0; i < nleaf; i++) {
    in >> level[i] >> org[3 * i] >> org[3 * i + 1] >> org[3 * i + 2];
    if (level[i] > max_level) max_level = level[i];
  }
  int nfaces = 0;
  in >> nfaces;
  std::vector<MhdRefreshFace> faces(nfaces);
  for (auto& f : faces)
    in >> f.sender >> f.receiver >> f.type >> f.face[0] >> f.face[1] >> f.face[2] >>
        f.child[0] >> f.child[1] >> f.child[2];
  if (!in) return fail("smr file");
  mhdvlct::EnzoMethodMHDVlctGB300 method(kHydroParams);
  const int m = n + 2 * g;
  const size_t M = (size_t)m * m * m, A = (size_t)n * n;
  const double pi = 3.14159265358979324, gam = 5.0 / 3.0;
  std::vector<mhdvlct::Block> blocks(nleaf);
  std::vector<MhdFluxCorrection> fluxes(nleaf);
  std::vector<void*> owned;
  std::vector<double> vol(nleaf);
  auto dev = [&](const std::vector<double>& v) {
    void* d = nullptr;
    cudaMalloc(&d, v.size() * sizeof(double));
    cudaMemcpy(d, v.data(), v.size() * sizeof(double), cudaMemcpyHostToDevice);
    owned.push_back(d);
    return d;
  };
  for (int i = 0; i < nleaf; i++) {
    const double h = 1.0 / (root * n) / (double)(1 << level[i]);
    const double hf = 1.0 / (root * n) / (double)(1 << max_level);
    vol[i] = h * h * h;
    std::vector<double> rho(M), v0(M, 0.4), v1(M, -0.3), v2(M, 0.2), e(M), p(M, 0.0);
    for (int z = 0; z < m; z++)
      for (int y = 0; y < m; y++)
        for (int x = 0; x < m; x++) {
          const double px = org[3 * i] * hf + (x - g + 0.5) * h;
          const double py = org[3 * i + 1] * hf + (y - g + 0.5) * h;
          const double pz = org[3 * i + 2] * hf + (z - g + 0.5) * h;
          const size_t c = ((size_t)z * m + y) * m + x;
          rho[c] = 1.0 + 0.5 * std::sin(2 * pi * (px + 2 * py + 3 * pz));
          e[c] = 0.6 / ((gam - 1.0) * rho[c]) + 0.5 * (0.16 + 0.09 + 0.04);
        }
    MhdBlockView& b = blocks[i].fields;
    std::memset(&b, 0, sizeof(b));
    b.dtype = MHD_DTYPE_F64;
    for (int a = 0; a < 3; a++) {
      b.n[a] = n;
      b.ghost[a] = g;
      b.cell_width[a] = h;
    }
    b.density = dev(rho);
    b.velocity[0] = dev(v0);
    b.velocity[1] = dev(v1);
    b.velocity[2] = dev(v2);
    b.total_energy = dev(e);
    b.pressure = dev(p);
    std::memset(&fluxes[i], 0, sizeof(fluxes[i]));
    for (int a = 0; a < 3; a++)
      for (int sd = 0; sd < 2; sd++)
        for (int q = 0; q < 5; q++) fluxes[i].flux[a][sd][q] = dev(std::vector<double>(A, 0.0));
  }
  auto totals = [&](long double out[2]) {
    out[0] = out[1] = 0.0L;
    std::vector<double> r(M), e(M);
    for (int i = 0; i < nleaf; i++) {
      cudaMemcpy(r.data(), blocks[i].fields.density, M * sizeof(double), cudaMemcpyDeviceToHost);
      cudaMemcpy(e.data(), blocks[i].fields.total_energy, M * sizeof(double),
                 cudaMemcpyDeviceToHost);
      for (int z = g; z < g + n; z++)
        for (int y = g; y < g + n; y++)
          for (int x = g; x < g + n; x++) {
            const size_t c = ((size_t)z * m + y) * m + x;
            out[0] += (long double)r[c] * vol[i];
            out[1] += (long double)r[c] * e[c] * vol[i];
          }
    }
  };
  method.refresh(blocks, faces);
  long double t0[2], t1[2];
  totals(t0);
  for (int cycle = 0; cycle < 2; cycle++) {
    double dt = 1e300;
    for (auto& b : blocks) dt = std::fmin(dt, method.timestep(b));
    method.refresh(blocks, faces);
    for (int i = 0; i < nleaf; i++) {
      blocks[i].dt = dt;
      method.compute_store_fluxes(blocks[i], fluxes[i]);
    }
    method.flux_correct(blocks, fluxes, faces);
  }
  totals(t1);
  for (void* d : owned) cudaFree(d);
  std::printf("smr ok: mass %.3Le energy %.3Le\n", fabsl(t1[0] - t0[0]) / fabsl(t0[0]),
              fabsl(t1[1] - t0[1]) / fabsl(t0[1]));
  return 0;
}

int main(int argc, char** argv) {
  if (argc > 2 && std::strcmp(argv[1], "--smr") == 0) {
    try {
      return run_smr(argv[2]);
    } catch (const mhdvlct::Error& e) {
      return fail(e.what());
    }
  }
  const bool gpu = argc > 1 && std::strcmp(argv[1], "--gpu") == 0;
  mhdvlct::EnzoMethodMHDVlctGB300 method(kParams);
  if (method.name() != "mhd_vlct") return fail("name");
  if (method.courant() != 0.4) return fail("courant");
  if (method.required_ghost_depth() != 3) return fail("ghost depth");
  // the reference's constructor errors become exceptions
  bool threw = false;
  try {
    mhdvlct::EnzoMethodMHDVlctGB300 bad(
        "Method { mhd_vlct { mhd_choice = \"constrained_transport\";"
        " riemann_solver = \"hllc\"; }; }");
  } catch (const mhdvlct::Error& e) {
    threw = e.code() == MHD_ERR_INVALID;
  }
  if (!threw) return fail("HLLC with constrained transport must be rejected");
  if (!gpu) {
    std::printf("cpp method ok (host)\n");
    return 0;
  }

  // one 8^3 block (3 ghosts) of a smooth MHD state, FP64
  const int n = 8, g = 3, m = n + 2 * g;
  const size_t M = (size_t)m * m * m, F = (size_t)(m + 1) * m * m;
  std::vector<double> h_c[9], h_f[3];
  for (auto& v : h_c) v.assign(M, 0.0);
  for (auto& v : h_f) v.assign(F, 0.0);
  const double bx0 = 0.3, by0 = 0.2, bz0 = 0.1, gam = 5.0 / 3.0;
  for (int z = 0; z < m; z++)
    for (int y = 0; y < m; y++)
      for (int x = 0; x < m; x++) {
        const size_t c = ((size_t)z * m + y) * m + x;
        const double rho = 1.0 + 0.1 * std::sin(0.7 * x + 0.3 * y + 0.2 * z);
        const double vx = 0.05 * std::cos(0.4 * y), vy = 0.03, vz = -0.02;
        const double p = 0.6;
        h_c[0][c] = rho;
        h_c[1][c] = vx;
        h_c[2][c] = vy;
        h_c[3][c] = vz;
        h_c[5][c] = bx0;
        h_c[6][c] = by0;
        h_c[7][c] = bz0;
        h_c[4][c] = p / ((gam - 1.0) * rho) + 0.5 * (vx * vx + vy * vy + vz * vz) +
                    0.5 * (bx0 * bx0 + by0 * by0 + bz0 * bz0) / rho;
      }
  for (auto& v : h_f) v.clear();
  h_f[0].assign((size_t)m * m * (m + 1), bx0);
  h_f[1].assign((size_t)m * (m + 1) * m, by0);
  h_f[2].assign((size_t)(m + 1) * m * m, bz0);

  auto upload = [](const std::vector<double>& v) {
    void* d = nullptr;
    cudaMalloc(&d, v.size() * sizeof(double));
    cudaMemcpy(d, v.data(), v.size() * sizeof(double), cudaMemcpyHostToDevice);
    return d;
  };
  mhdvlct::Block blocks[2];
  std::vector<void*> owned;
  for (auto& b : blocks) {
    std::memset(&b.fields, 0, sizeof(b.fields));
    b.fields.dtype = MHD_DTYPE_F64;
    for (int a = 0; a < 3; a++) {
      b.fields.n[a] = n;
      b.fields.ghost[a] = g;
      b.fields.cell_width[a] = 1.0 / n;
    }
    b.fields.density = upload(h_c[0]);
    for (int a = 0; a < 3; a++) b.fields.velocity[a] = upload(h_c[1 + a]);
    b.fields.total_energy = upload(h_c[4]);
    for (int a = 0; a < 3; a++) b.fields.bfield[a] = upload(h_c[5 + a]);
    for (int a = 0; a < 3; a++) b.fields.bfieldi[a] = upload(h_f[a]);
    b.fields.pressure = upload(std::vector<double>(M, 0.0));
    owned.insert(owned.end(), {b.fields.density, b.fields.velocity[0], b.fields.velocity[1],
                               b.fields.velocity[2], b.fields.total_energy,
                               b.fields.bfield[0], b.fields.bfield[1], b.fields.bfield[2],
                               b.fields.bfieldi[0], b.fields.bfieldi[1], b.fields.bfieldi[2],
                               b.fields.pressure});
  }
  // block 0 through the C++ Method, block 1 through the plain C ABI
  method.refresh_periodic(blocks[0]);
  blocks[0].dt = method.timestep(blocks[0]);
  method.compute(blocks[0]);
  MhdVlctParams p;
  char err[256];
  if (mhdvlct_params_parse(kParams, &p, err, sizeof(err)) != MHD_OK) return fail(err);
  mhdvlct_handle* h = nullptr;
  if (mhdvlct_create(&p, &h) != MHD_OK) return fail("create");
  double dt = 0;
  if (mhdvlct_fill_ghosts_periodic(h, &blocks[1].fields, nullptr) != MHD_OK ||
      mhdvlct_block_timestep(h, &blocks[1].fields, &dt, nullptr) != MHD_OK ||
      mhdvlct_block_step(h, &blocks[1].fields, dt, nullptr) != MHD_OK)
    return fail(mhdvlct_last_error_string(h));
  mhdvlct_destroy(h);
  if (dt != blocks[0].dt) return fail("dt differs");
  std::vector<double> a(M), b(M);
  cudaMemcpy(a.data(), blocks[0].fields.density, M * sizeof(double), cudaMemcpyDeviceToHost);
  cudaMemcpy(b.data(), blocks[1].fields.density, M * sizeof(double), cudaMemcpyDeviceToHost);
  if (a != b) return fail("density differs");
  bool changed = false;
  for (size_t i = 0; i < M; i++) changed = changed || a[i] != h_c[0][i];
  if (!changed) return fail("the step did not change the density");
  for (void* d : owned) cudaFree(d);
  std::printf("cpp method ok (gpu): dt %.17g\n", dt);
  return 0;
}
