// capi.cu -- C ABI: parameters, handle and the per-block Method operations
// (EnzoMethodMHDVlct::compute / ::timestep and the ghost refresh), with the
// optional gravity source, passive scalars and flux-correction output, and
// the no-allocation variant of the step.
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <mutex>
#include <vector>

#include "capi_internal.h"
#include "vlct_aux.cuh"

using namespace vlct;

static_assert(kFluxQuantities == MHD_FC_NQ, "flux-correction quantity slots");

namespace mhdint {

int fail(mhdvlct_handle* h, int code, const std::string& msg) {
  if (h) h->err = msg;
  return code;
}

static std::string lower(const char* s) {
  std::string o(s ? s : "");
  for (auto& c : o) c = (char)std::tolower((unsigned char)c);
  return o;
}

StagePlan stage_plan(const mhdvlct_handle* h) {
  StagePlan p;
  auto imm = [](int r) { return r == RECON_NN ? 0 : 1; };
  auto tot = [](int r) { return r == RECON_NN ? 1 : 2; };
  if (h->euler) {
    p.nstages = 1;
    p.recon[0] = h->recon;
    p.s[0] = 0;
    p.S[0] = imm(h->recon);
    p.dt_factor[0] = 1.0;
  } else {
    p.nstages = 2;
    p.recon[0] = RECON_NN;
    p.recon[1] = h->recon;
    p.s[0] = 0;
    p.S[0] = 0;
    p.dt_factor[0] = 0.5;
    p.s[1] = tot(RECON_NN);
    p.S[1] = p.s[1] + imm(h->recon);
    p.dt_factor[1] = 1.0;
  }
  return p;
}

// near-equal split of [lo, hi) into parts of at most t
static void split(int lo, int hi, int t, std::vector<std::pair<int, int>>& out) {
  out.clear();
  const int len = hi - lo;
  if (len <= 0) return;
  if (t <= 0 || t > len) t = len;
  const int n = (len + t - 1) / t;
  int a = lo;
  for (int i = 0; i < n; i++) {
    const int w = len / n + (i < len % n ? 1 : 0);
    out.push_back({a, a + w});
    a += w;
  }
}

void make_tiles(int block, const int m[3], int S, bool final, int tile_x,
                int tile_y, int zchunk, std::vector<StageTile>& out) {
  const int lo = final ? S : S + 1;
  const int hi_x = final ? m[0] - S : m[0] - S - 1;
  const int hi_y = final ? m[1] - S : m[1] - S - 1;
  const int hi_z = final ? m[2] - S : m[2] - S - 1;
  std::vector<std::pair<int, int>> xs, ys, zs;
  split(lo, hi_x, tile_x, xs);
  split(lo, hi_y, tile_y, ys);
  split(lo, hi_z, zchunk > 0 ? zchunk : (hi_z - lo), zs);
  for (auto& z : zs)
    for (auto& y : ys)
      for (auto& x : xs)
        out.push_back({block, x.first, x.second, y.first, y.second, z.first, z.second});
}

template <class R>
FieldSet<R> fieldset_of(const MhdBlockView* b) {
  FieldSet<R> f;
  f.c[F_RHO] = (R*)b->density;
  f.c[F_VX] = (R*)b->velocity[0];
  f.c[F_VY] = (R*)b->velocity[1];
  f.c[F_VZ] = (R*)b->velocity[2];
  f.c[F_ETOT] = (R*)b->total_energy;
  f.c[F_EINT] = (R*)b->internal_energy;
  f.c[F_BX] = (R*)b->bfield[0];
  f.c[F_BY] = (R*)b->bfield[1];
  f.c[F_BZ] = (R*)b->bfield[2];
  for (int d = 0; d < 3; d++) f.f[d] = (R*)b->bfieldi[d];
  return f;
}
template FieldSet<double> fieldset_of<double>(const MhdBlockView*);
template FieldSet<float> fieldset_of<float>(const MhdBlockView*);

int default_tile(int dtype, int solver, int recon, int de) {
  // largest square tile whose shared memory fits the CTAs an SM holds at
  // once (227 KB per SM): one CTA for FP64, three for the FP32 NN stage, two
  // for the other FP32 stages
  const int cap = (dtype == MHD_DTYPE_F64) ? 200 * 1024
                  : (recon == RECON_NN)    ? 72 * 1024
                                           : 110 * 1024;
  int best = 4;
  for (int t = 4; t <= (dtype == MHD_DTYPE_F64 ? TileLimits<double>::TMAX
                                                 : TileLimits<float>::TMAX);
       t++) {
    const size_t b = (dtype == MHD_DTYPE_F64)
                         ? stage_smem<double>(solver, recon, de != 0, t, t)
                         : stage_smem<float>(solver, recon, de != 0, t, t);
    if (b <= (size_t)cap) best = t;
  }
  return best;
}

void default_tile_xy(int dtype, int solver, int recon, int de, int& tx, int& ty) {
  if (dtype == MHD_DTYPE_F32) {
    // the shapes the autotuner settles on for 32^3 blocks: wide in x
    // (coalesced rows), one large tile per SM; the tile split evens them
    // out over other block sizes.  Both fit 227 KB with dual energy.
    tx = recon == RECON_NN ? 34 : 24;
    ty = recon == RECON_NN ? 10 : 16;
    return;
  }
  tx = ty = default_tile(dtype, solver, recon, de);
}

}  // namespace mhdint

using namespace mhdint;

// ------------------------------------------------------------------ params
extern "C" void mhdvlct_params_default(MhdVlctParams* p) {
  std::memset(p, 0, sizeof(*p));
  std::snprintf(p->riemann_solver, sizeof(p->riemann_solver), "hlld");
  std::snprintf(p->time_scheme, sizeof(p->time_scheme), "vl");
  std::snprintf(p->reconstruct_method, sizeof(p->reconstruct_method), "plm");
  p->theta_limiter = 1.5;
  p->courant = -1.0;  // resolved from time_scheme at create (vl: 0.3, euler: 1)
  p->gamma = 5.0 / 3.0;
  p->density_floor = 0.0;
  p->pressure_floor = 0.0;
  p->dual_energy = 0;
  p->dual_energy_eta = 0.001;
}

namespace {
// Minimal reader of the Cello parameter language subset used by this
// method: nested groups `Name { ... }`, assignments `key = value;` with
// string, number or logical values.  Produces dotted paths such as
// "Method:mhd_vlct:riemann_solver".
struct PTok {
  std::string path, value;
  bool is_string;
};
static bool parse_params(const char* text, std::vector<PTok>& out,
                         std::string& err) {
  std::vector<std::string> stack;
  const char* c = text;
  auto skip = [&]() {
    for (;;) {
      while (*c && std::isspace((unsigned char)*c)) c++;
      if (*c == '#') {
        while (*c && *c != '\n') c++;
        continue;
      }
      break;
    }
  };
  std::string pending;
  for (;;) {
    skip();
    if (!*c) break;
    if (*c == '}') {
      if (stack.empty()) { err = "unbalanced '}'"; return false; }
      stack.pop_back();
      c++;
      skip();
      if (*c == ';') c++;
      continue;
    }
    if (*c == ';') { c++; continue; }
    const char* s0 = c;
    while (*c && (std::isalnum((unsigned char)*c) || *c == '_' || *c == ':')) c++;
    std::string ident(s0, c);
    if (ident.empty()) { err = std::string("unexpected character '") + *c + "'"; return false; }
    skip();
    if (*c == '{') {
      stack.push_back(ident);
      c++;
      continue;
    }
    if (*c != '=') { err = "expected '=' after " + ident; return false; }
    c++;
    skip();
    PTok t;
    std::string path;
    for (auto& s : stack) path += s + ":";
    t.path = path + ident;
    t.is_string = false;
    if (*c == '"') {
      c++;
      const char* v0 = c;
      while (*c && *c != '"') c++;
      if (*c != '"') { err = "unterminated string"; return false; }
      t.value.assign(v0, c);
      t.is_string = true;
      c++;
    } else if (*c == '[') {  // lists are skipped
      int depth = 0;
      do {
        if (*c == '[') depth++;
        if (*c == ']') depth--;
        c++;
      } while (*c && depth > 0);
    } else {
      const char* v0 = c;
      while (*c && *c != ';' && *c != '}' && !std::isspace((unsigned char)*c)) c++;
      t.value.assign(v0, c);
    }
    skip();
    if (*c == ';') c++;
    out.push_back(t);
  }
  if (!stack.empty()) { err = "unbalanced '{'"; return false; }
  return true;
}
}  // namespace

extern "C" int mhdvlct_params_parse(const char* text, MhdVlctParams* out,
                                    char* errbuf, size_t errbuf_len) {
  auto report = [&](const std::string& m) {
    if (errbuf && errbuf_len) std::snprintf(errbuf, errbuf_len, "%s", m.c_str());
    return MHD_ERR_INVALID;
  };
  if (!text || !out) return report("null argument");
  mhdvlct_params_default(out);
  std::vector<PTok> toks;
  std::string err;
  if (!parse_params(text, toks, err)) return report(err);
  for (const auto& t : toks) {
    const std::string& k = t.path;
    auto num = [&](double* dst) -> bool {
      char* end = nullptr;
      const double v = std::strtod(t.value.c_str(), &end);
      if (!end || *end) return false;
      *dst = v;
      return true;
    };
    auto str = [&](char* dst, size_t n) -> bool {
      if (!t.is_string || t.value.size() + 1 > n) return false;
      std::snprintf(dst, n, "%s", t.value.c_str());
      return true;
    };
    bool ok = true;
    if (k == "Method:mhd_vlct:mhd_choice") ok = str(out->mhd_choice, sizeof(out->mhd_choice));
    else if (k == "Method:mhd_vlct:riemann_solver") ok = str(out->riemann_solver, sizeof(out->riemann_solver));
    else if (k == "Method:mhd_vlct:time_scheme") ok = str(out->time_scheme, sizeof(out->time_scheme));
    else if (k == "Method:mhd_vlct:reconstruct_method") ok = str(out->reconstruct_method, sizeof(out->reconstruct_method));
    else if (k == "Method:mhd_vlct:theta_limiter") ok = num(&out->theta_limiter);
    else if (k == "Method:mhd_vlct:courant") ok = num(&out->courant);
    else if (k == "Physics:fluid_props:eos:gamma") ok = num(&out->gamma);
    else if (k == "Physics:fluid_props:floors:density") ok = num(&out->density_floor);
    else if (k == "Physics:fluid_props:floors:pressure") ok = num(&out->pressure_floor);
    else if (k == "Physics:fluid_props:dual_energy:eta") ok = num(&out->dual_energy_eta);
    else if (k == "Physics:fluid_props:dual_energy:type") {
      const std::string v = lower(t.value.c_str());
      if (v == "modern") out->dual_energy = 1;
      else if (v == "disabled" || v == "none") out->dual_energy = 0;
      else return report("dual_energy:type \"" + t.value + "\" is not supported");
    } else if (k == "Method:mhd_vlct:half_dt_reconstruct_method" ||
               k == "Method:mhd_vlct:full_dt_reconstruct_method") {
      // removed parameters (EnzoMethodMHDVlct.cpp:62-70)
      return report(k + " has been removed; use reconstruct_method");
    }
    if (!ok) return report("bad value for " + k + ": " + t.value);
  }
  return MHD_OK;
}

// ------------------------------------------------------------------ handle
extern "C" int mhdvlct_create(const MhdVlctParams* p, mhdvlct_handle** out) {
  if (!p || !out) return MHD_ERR_INVALID;
  *out = nullptr;
  mhdvlct_handle* h = new mhdvlct_handle();
  h->params = *p;
  auto bad = [&](const std::string& m) {
    // keep the handle so the caller can read the message, but signal failure
    h->err = m;
    *out = h;
    return MHD_ERR_INVALID;
  };
  const std::string choice = lower(p->mhd_choice);
  if (choice.empty()) return bad("Method:mhd_vlct:mhd_choice wasn't specified");
  if (choice == "no_bfield") h->mhd = 0;
  else if (choice == "constrained_transport") h->mhd = 1;
  else if (choice == "unsafe_constant_uniform")
    return bad("unsafe_constant_uniform is for debugging only and is not supported");
  else return bad("Unrecognized mhd_choice \"" + std::string(p->mhd_choice) + "\"");
  // EnzoRiemann::construct_riemann (riemann/EnzoRiemann.cpp:26-68)
  const std::string rs = lower(p->riemann_solver);
  if (rs == "hlld") {
    if (!h->mhd) return bad("The \"HLLD\" Riemann Solver requires magnetic fields");
    h->solver = SOLVER_HLLD;
  } else if (rs == "hlle") {
    if (!h->mhd) return bad("The \"HLLE\" Riemann solver without magnetic fields is untested");
    h->solver = SOLVER_HLLE;
  } else if (rs == "hllc") {
    if (h->mhd) return bad("The \"HLLC\" Riemann Solver can't support mhd");
    h->solver = SOLVER_HLLC;
  } else if (rs == "hll") {
    return bad("The \"HLL\" (Davis wave speed) solver is untested in the reference");
  } else {
    return bad("The only known solvers are HLL, HLLE, HLLC, & HLLD");
  }
  // EnzoReconstructor::construct_reconstructor (toolkit/EnzoReconstructor.cpp:14-44)
  if (!(1. <= p->theta_limiter && p->theta_limiter <= 2.))
    return bad("theta_limiter must satisfy 1<=theta_limiter<=2");
  const std::string rc = lower(p->reconstruct_method);
  if (rc == "nn") h->recon = RECON_NN;
  else if (rc == "plm" || rc == "plm_enzo") h->recon = RECON_PLM;
  else if (rc == "plm_athena") h->recon = RECON_PLM_ATHENA;
  else return bad("The only allowed reconstructors are NN, PLM, PLM_ENZO, & PLM_ATHENA");
  const std::string ts = lower(p->time_scheme);
  if (ts == "vl") h->euler = 0;
  else if (ts == "euler") h->euler = 1;
  else return bad("time_scheme must be \"vl\" or \"euler\"");
  // EnzoBfieldMethod::EnzoBfieldMethod (toolkit/EnzoBfieldMethod.cpp:15-28):
  // constrained transport with one partial timestep is an ERROR
  if (h->euler && h->mhd)
    return bad("constrained_transport hasn't been tested for num_partial_timesteps != 2 "
               "(time_scheme \"euler\" needs mhd_choice \"no_bfield\")");
  if (h->params.courant < 0) h->params.courant = h->euler ? 1.0 : 0.3;
  if (!(p->gamma > 1.0)) return bad("gamma should exceed 1.0");
  // EnzoMHDIntegratorStageCommands ctor (EnzoMHDIntegratorStageCommands.cpp:35-40)
  if (!(p->density_floor > 0) || !(p->pressure_floor > 0))
    return bad("density and pressure floors must be defined");
  h->de = p->dual_energy ? 1 : 0;
  if (h->de && !(p->dual_energy_eta >= 0)) return bad("eta must be non-negative");
  h->phys.gamma = p->gamma;
  h->phys.density_floor = p->density_floor;
  h->phys.pressure_floor = p->pressure_floor;
  h->phys.theta_limiter = p->theta_limiter;
  h->phys.eta = h->de ? p->dual_energy_eta : 0.0;
  h->phys.set_derived();
  *out = h;
  return MHD_OK;
}

extern "C" int mhdvlct_destroy(mhdvlct_handle* h) {
  if (!h) return MHD_ERR_INVALID;
  if (h->scratch) cudaFree(h->scratch);
  if (h->rf_dev) cudaFree(h->rf_dev);
  if (h->rf_done) cudaEventDestroy(h->rf_done);
  delete h;
  return MHD_OK;
}

extern "C" const char* mhdvlct_last_error_string(const mhdvlct_handle* h) {
  return h ? h->err.c_str() : "null handle";
}

extern "C" double mhdvlct_courant(const mhdvlct_handle* h) {
  return h ? h->params.courant : -1.0;
}

extern "C" int mhdvlct_required_ghost_depth(const mhdvlct_handle* h) {
  if (!h) return -1;
  const StagePlan sp = stage_plan(h);
  int g = 0;
  for (int i = 0; i < sp.nstages; i++) g += (sp.recon[i] == RECON_NN) ? 1 : 2;
  return g;
}

// -------------------------------------------------------------- one block
namespace {

int check_view(mhdvlct_handle* h, const MhdBlockView* b) {
  if (!b) return fail(h, MHD_ERR_INVALID, "null block view");
  if (b->dtype != MHD_DTYPE_F64 && b->dtype != MHD_DTYPE_F32)
    return fail(h, MHD_ERR_INVALID, "unknown dtype");
  if (b->ghost[0] != b->ghost[1] || b->ghost[0] != b->ghost[2])
    return fail(h, MHD_ERR_INVALID, "ghost depth must be equal on all axes");
  if (b->ghost[0] < mhdvlct_required_ghost_depth(h))
    return fail(h, MHD_ERR_GHOST,
                "ghost depth must be at least " +
                    std::to_string(mhdvlct_required_ghost_depth(h)));
  for (int a = 0; a < 3; a++) {
    if (b->n[a] < 1) return fail(h, MHD_ERR_INVALID, "block extents must be positive");
    if (!(b->cell_width[a] > 0)) return fail(h, MHD_ERR_INVALID, "cell widths must be positive");
    if (b->n[a] + 2 * b->ghost[a] > 4096) return fail(h, MHD_ERR_INVALID, "block too large");
  }
  if (!b->density || !b->velocity[0] || !b->velocity[1] || !b->velocity[2] ||
      !b->total_energy)
    return fail(h, MHD_ERR_INVALID, "missing hydro field pointer");
  if (h->de && !b->internal_energy)
    return fail(h, MHD_ERR_INVALID, "internal_energy is required with dual energy");
  if (h->mhd) {
    for (int d = 0; d < 3; d++)
      if (!b->bfield[d] || !b->bfieldi[d])
        return fail(h, MHD_ERR_INVALID, "missing bfield / bfieldi pointer");
  }
  const int nacc = (b->acceleration[0] != nullptr) + (b->acceleration[1] != nullptr) +
                   (b->acceleration[2] != nullptr);
  if (nacc != 0 && nacc != 3)
    return fail(h, MHD_ERR_INVALID, "give all three acceleration fields or none");
  if (b->npassive < 0 || b->npassive > 4)
    return fail(h, MHD_ERR_INVALID, "npassive must be in [0, 4]");
  for (int k = 0; k < b->npassive; k++)
    if (!b->passive[k]) return fail(h, MHD_ERR_INVALID, "missing passive scalar pointer");
  return MHD_OK;
}

int cuda_fail(mhdvlct_handle* h, cudaError_t e, const char* where) {
  return fail(h, MHD_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

// Descriptor uploads go through a kernel parameter instead of a
// cudaMemcpyAsync from host memory: a copy from pageable memory may make the
// host wait for the stream, so consecutive per-block calls would no longer
// queue behind each other.  The bytes are passed by value in chunks.
constexpr int kBlobBytes = 1024;
struct Blob {
  unsigned char b[kBlobBytes];
};
__global__ void put_blob_kernel(unsigned char* dst, Blob src, int n) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = src.b[i];
}
cudaError_t put_bytes(void* dst, const void* src, size_t n, cudaStream_t st) {
  const unsigned char* s = (const unsigned char*)src;
  for (size_t off = 0; off < n; off += kBlobBytes) {
    const int k = (int)std::min<size_t>(kBlobBytes, n - off);
    Blob bl;
    std::memcpy(bl.b, s + off, k);
    put_blob_kernel<<<1, 128, 0, st>>>((unsigned char*)dst + off, bl, k);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// Cello's min-reduction of the blocks' dt (control_stopping.cpp:96-106) on
// the device: one CTA, a min is exact in any order.
__global__ void dt_min_kernel(const double* v, int n, double* out) {
  __shared__ double red[256];
  double m = v[0];
  for (int i = threadIdx.x; i < n; i += blockDim.x) m = (v[i] < m) ? v[i] : m;
  red[threadIdx.x] = m;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      const double o = red[threadIdx.x + w];
      if (o < red[threadIdx.x]) red[threadIdx.x] = o;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = red[0];
}
cudaError_t launch_dt_min(const double* v, int n, double* out, cudaStream_t st) {
  dt_min_kernel<<<1, 256, 0, st>>>(v, n, out);
  return cudaGetLastError();
}

// The tiles of make_tiles (same near-equal split of each axis, same order:
// x fastest, then y, then z), generated on the device: tile i of
// nx * ny * nz parts of the output window [lo, hi_a) of each axis a.
struct TileSplit {
  int block, lo, len[3], np[3];
};
__global__ void make_tiles_kernel(StageTile* out, TileSplit sp) {
  const int n = sp.np[0] * sp.np[1] * sp.np[2];
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    int q[3] = {t % sp.np[0], (t / sp.np[0]) % sp.np[1], t / (sp.np[0] * sp.np[1])};
    int a0[3], a1[3];
    for (int a = 0; a < 3; a++) {
      const int base = sp.len[a] / sp.np[a], rem = sp.len[a] % sp.np[a];
      a0[a] = sp.lo + q[a] * base + (q[a] < rem ? q[a] : rem);
      a1[a] = a0[a] + base + (q[a] < rem ? 1 : 0);
    }
    out[t] = StageTile{sp.block, a0[0], a1[0], a0[1], a1[1], a0[2], a1[2]};
  }
}
// The split of one stage's output window into tiles of at most tx x ty
// columns and z-chunks of zchunk planes (0: whole window); ntiles() = 0 when
// the window is empty.
TileSplit tile_split(const int m[3], int S, bool final, int tx, int ty, int zchunk) {
  TileSplit sp{};
  sp.lo = final ? S : S + 1;
  const int t[3] = {tx, ty, zchunk};
  for (int a = 0; a < 3; a++) {
    sp.len[a] = (final ? m[a] - S : m[a] - S - 1) - sp.lo;
    int ta = t[a];
    if (sp.len[a] <= 0) {
      sp.np[0] = sp.np[1] = sp.np[2] = 0;
      return sp;
    }
    if (ta <= 0 || ta > sp.len[a]) ta = sp.len[a];
    sp.np[a] = (sp.len[a] + ta - 1) / ta;
  }
  return sp;
}
long ntiles_of(const TileSplit& sp) { return (long)sp.np[0] * sp.np[1] * sp.np[2]; }
cudaError_t launch_make_tiles(StageTile* out, const TileSplit& sp, cudaStream_t st) {
  const long n = ntiles_of(sp);
  if (n <= 0) return cudaSuccess;
  make_tiles_kernel<<<(int)std::min<long>((n + 127) / 128, 64), 128, 0, st>>>(out, sp);
  return cudaGetLastError();
}

// Work decomposition of one stage of the per-block path: the tile extent and
// z-chunk that minimise a simple cost model for one block alone on the GPU.
// A tile of t x t columns and L planes costs about (t+2)^2 (L + 1.5) (its
// halo columns and the planes of its prologue); the tiles run in waves of
// the CTAs the GPU holds at once (one per SM for FP64, two or three for
// FP32), so the stage takes about waves x the largest tile's cost.
struct PlainDecomp {
  int tile[2] = {8, 8};
  int zchunk[2] = {0, 0};
};
int sm_count() {
  static const int n = [] {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0)
      v = 1;
    return v;
  }();
  return n;
}
PlainDecomp plain_decomp(const mhdvlct_handle* h, const int m[3], int dtype) {
  PlainDecomp d;
  const StagePlan sp = stage_plan(h);
  for (int i = 0; i < sp.nstages; i++) {
    const bool final = i + 1 == sp.nstages;
    const int tmax = default_tile(dtype, h->solver, sp.recon[i], h->de);
    const int per_sm = dtype == MHD_DTYPE_F64 ? 1 : (sp.recon[i] == RECON_NN) ? 3 : 2;
    const long resident = (long)per_sm * sm_count();
    double best = 1e300;
    for (int t = std::min(6, tmax); t <= tmax; t++) {
      for (int L : {0, 16, 12, 8, 6, 4}) {
        const TileSplit s = tile_split(m, sp.S[i], final, t, t, L);
        const long n = ntiles_of(s);
        if (n <= 0) continue;
        const int tx = (s.len[0] + s.np[0] - 1) / s.np[0];
        const int ty = (s.len[1] + s.np[1] - 1) / s.np[1];
        const int tz = (s.len[2] + s.np[2] - 1) / s.np[2];
        const double cost = (double)((n + resident - 1) / resident) * (tx + 2) * (ty + 2) *
                            (tz + 1.5);
        if (cost < best * 0.999) {  // on ties the smaller tile / fewer chunks stays
          best = cost;
          d.tile[i] = t;
          d.zchunk[i] = L;
        }
      }
    }
    if (h->tile > 0) d.tile[i] = h->tile;  // a tile set on the handle wins
    if (h->zchunk > 0) d.zchunk[i] = h->zchunk;
  }
  return d;
}

// Scratch of the plain path, carved from one allocation.
template <class R> struct PlainScratch {
  R* tmp[NCELL];
  R* tpass[4];               // half-step passive scalars
  R* dflux[3];               // with passive scalars: the stages' density fluxes
  R* tface[3];
  R* fface[3];
  double* d_dt;
  double* d_dtout;
  void* d_smax;
  StageBlock<R>* d_sblocks;  // [2]
  AuxBlock<R>* d_aux;        // [1]
  int* d_nbr;                // [27]
  void* d_fc;                // FluxOut<R> for the boundary fluxes
  StageTile* d_tiles;        // stage 0 tiles then stage 1 tiles
  int ntiles[2];
  int tile[2];               // largest tile extent of each stage
};

size_t align_up(size_t v) { return (v + 255) & ~(size_t)255; }

template <class R>
int ensure_scratch(mhdvlct_handle* h, const int m[3], int dtype,
                   PlainScratch<R>& S, cudaStream_t st, int np = 0) {
  const StagePlan sp = stage_plan(h);
  const PlainDecomp dc = plain_decomp(h, m, dtype);
  TileSplit ts[2] = {};
  long nt[2] = {0, 0};
  for (int i = 0; i < sp.nstages; i++) {
    ts[i] = tile_split(m, sp.S[i], i + 1 == sp.nstages, dc.tile[i], dc.tile[i], dc.zchunk[i]);
    nt[i] = ntiles_of(ts[i]);
  }
  const size_t M = (size_t)m[0] * m[1] * m[2];
  const size_t F[3] = {(size_t)(m[0] + 1) * m[1] * m[2],
                       (size_t)m[0] * (m[1] + 1) * m[2],
                       (size_t)m[0] * m[1] * (m[2] + 1)};
  size_t off = 0;
  std::vector<size_t> offs;
  auto take = [&](size_t bytes) { offs.push_back(off); off += align_up(bytes); };
  for (int k = 0; k < NCELL; k++) take(M * sizeof(R));
  for (int d = 0; d < 3; d++) take(F[d] * sizeof(R));
  for (int d = 0; d < 3; d++) take(F[d] * sizeof(R));
  for (int k = 0; k < np; k++) take(M * sizeof(R));
  for (int d = 0; d < 3 && np > 0; d++) take(M * sizeof(R));
  take(sizeof(double));
  take(sizeof(double));
  take(3 * sizeof(unsigned long long));
  take(2 * sizeof(StageBlock<R>));
  take(sizeof(AuxBlock<R>));
  take(27 * sizeof(int));
  take(sizeof(FluxOut<R>));
  take((size_t)(nt[0] + nt[1]) * sizeof(StageTile));
  const bool same = h->scratch && h->cache_dtype == dtype && h->cache_m[0] == m[0] &&
                    h->cache_m[1] == m[1] && h->cache_m[2] == m[2] &&
                    h->cache_np == np && h->scratch_bytes >= off;
  if (!same) {
    if (h->scratch) {
      cudaStreamSynchronize(st);
      cudaFree(h->scratch);
      h->scratch = nullptr;
    }
    cudaError_t e = cudaMalloc(&h->scratch, off);
    if (e != cudaSuccess) {
      h->scratch = nullptr;
      return fail(h, MHD_ERR_NOMEM, std::string("scratch allocation: ") + cudaGetErrorString(e));
    }
    h->scratch_bytes = off;
    h->cache_dtype = dtype;
    h->cache_np = np;
    for (int a = 0; a < 3; a++) h->cache_m[a] = m[a];
  }
  char* base = (char*)h->scratch;
  int i = 0;
  for (int k = 0; k < NCELL; k++) S.tmp[k] = (R*)(base + offs[i++]);
  for (int d = 0; d < 3; d++) S.tface[d] = (R*)(base + offs[i++]);
  for (int d = 0; d < 3; d++) S.fface[d] = (R*)(base + offs[i++]);
  for (int k = 0; k < 4; k++) S.tpass[k] = k < np ? (R*)(base + offs[i++]) : nullptr;
  for (int d = 0; d < 3; d++) S.dflux[d] = np > 0 ? (R*)(base + offs[i++]) : nullptr;
  S.d_dt = (double*)(base + offs[i++]);
  S.d_dtout = (double*)(base + offs[i++]);
  S.d_smax = (void*)(base + offs[i++]);
  S.d_sblocks = (StageBlock<R>*)(base + offs[i++]);
  S.d_aux = (AuxBlock<R>*)(base + offs[i++]);
  S.d_nbr = (int*)(base + offs[i++]);
  S.d_fc = (void*)(base + offs[i++]);
  S.d_tiles = (StageTile*)(base + offs[i++]);
  S.ntiles[0] = (int)nt[0];
  S.ntiles[1] = (int)nt[1];
  S.tile[0] = dc.tile[0];
  S.tile[1] = dc.tile[1];
  if (!same) {
    cudaError_t e = launch_make_tiles(S.d_tiles, ts[0], st);
    if (e == cudaSuccess) e = launch_make_tiles(S.d_tiles + nt[0], ts[1], st);
    if (e != cudaSuccess) return cuda_fail(h, e, "tile set-up");
    // a single block refreshes from itself: every neighbour entry is 0
    e = cudaMemsetAsync(S.d_nbr, 0, 27 * sizeof(int), st);
    if (e != cudaSuccess) return cuda_fail(h, e, "neighbour set-up");
    // scratch cell fields that a block never writes must still be defined
    e = cudaMemsetAsync(h->scratch, 0, offs[NCELL + 6 + np], st);
    if (e != cudaSuccess) return cuda_fail(h, e, "scratch clear");
  }
  return MHD_OK;
}

// One block step on scratch S, whose tiles are in place: the stage
// descriptors, the euler copy, both stages and the face copy-back.  dt is
// read on the device from d_dt.  Shared by the allocating and the
// no-allocation entry points.
template <class R>
int block_step_on(mhdvlct_handle* h, const MhdBlockView* b, PlainScratch<R>& S,
                  const double* d_dt, const MhdFluxCorrection* fc, cudaStream_t st) {
  const int g = b->ghost[0];
  const int m[3] = {b->n[0] + 2 * g, b->n[1] + 2 * g, b->n[2] + 2 * g};
  const int np = b->npassive;
  const StagePlan sp = stage_plan(h);
  FieldSet<R> ext = fieldset_of<R>(b);
  FieldSet<R> tmp;
  for (int k = 0; k < NCELL; k++) tmp.c[k] = S.tmp[k];
  for (int d = 0; d < 3; d++) tmp.f[d] = S.tface[d];
  const size_t M = (size_t)m[0] * m[1] * m[2];
  cudaError_t e;

  StageBlock<R> sb[2];
  for (int i = 0; i < sp.nstages; i++) {
    StageBlock<R>& B = sb[i];
    for (int a = 0; a < 3; a++) {
      B.m[a] = m[a];
      B.cw[a] = b->cell_width[a];
    }
    B.dt = d_dt;
    const bool final = (i + 1) == sp.nstages;
    B.base = ext;
    for (int d = 0; d < 3; d++) B.accel[d] = (const R*)b->acceleration[d];
    for (int k = 0; k < np; k++) {
      R* ep = (R*)b->passive[k];
      B.pass_base[k] = ep;
      // vl: stage 0 reads the caller's scalars and writes the half step,
      // stage 1 reads the half step and writes the caller's; euler reads a
      // copy (made below) and writes the caller's
      B.pass_cur[k] = (sp.nstages == 1 || i == 1) ? S.tpass[k] : ep;
      B.pass_out[k] = (sp.nstages == 2 && i == 0) ? S.tpass[k] : ep;
    }
    for (int d = 0; d < 3; d++) B.dflux[d] = np > 0 ? S.dflux[d] : nullptr;
    if (sp.nstages == 1) {
      // euler: a single stage cannot update its own input in place, so it
      // reads a copy of the block and writes into the caller's fields
      B.cur = tmp;
      for (int d = 0; d < 3; d++) B.cur.f[d] = ext.f[d];
      B.out = ext;
    } else if (i == 0) {
      B.cur = ext;
      B.out = tmp;
    } else {
      B.cur = tmp;
      B.out = ext;
    }
    if (final) {
      for (int d = 0; d < 3; d++) B.out.f[d] = S.fface[d];
    }
  }
  e = put_bytes(S.d_sblocks, sb, sizeof(sb), st);
  if (e != cudaSuccess) return cuda_fail(h, e, "block upload");
  if (fc) {
    FluxOut<R> fo;
    for (int d = 0; d < 3; d++)
      for (int sd = 0; sd < 2; sd++)
        for (int q = 0; q < kFluxQuantities; q++) fo.f[d][sd][q] = (R*)fc->flux[d][sd][q];
    fo.g = b->ghost[0];
    e = put_bytes(S.d_fc, &fo, sizeof(fo), st);
    if (e != cudaSuccess) return cuda_fail(h, e, "flux buffer upload");
  }
  if (sp.nstages == 1) {
    for (int k = 0; k < NCELL; k++) {
      if (!ext.c[k]) continue;
      e = cudaMemcpyAsync(S.tmp[k], ext.c[k], M * sizeof(R), cudaMemcpyDeviceToDevice, st);
      if (e != cudaSuccess) return cuda_fail(h, e, "euler copy");
    }
    for (int k = 0; k < np; k++) {
      e = cudaMemcpyAsync(S.tpass[k], b->passive[k], M * sizeof(R), cudaMemcpyDeviceToDevice,
                          st);
      if (e != cudaSuccess) return cuda_fail(h, e, "euler copy");
    }
  }
  const StageTile* tiles[2] = {S.d_tiles, S.d_tiles + S.ntiles[0]};
  for (int i = 0; i < sp.nstages; i++) {
    StageInfo info;
    info.s = sp.s[i];
    info.S = sp.S[i];
    info.final_stage = (i + 1) == sp.nstages;
    info.dt_factor = sp.dt_factor[i];
    info.tx = S.tile[i];
    info.ty = S.tile[i];
    info.queue = nullptr;
    info.threads = 256;
    // EnzoMHDIntegratorStageCommands.cpp:279: the gravity source enters the
    // stage with index 1 (the full-dt stage of vl; never with euler)
    info.gravity = (i == 1 && b->acceleration[0] != nullptr) ? 1 : 0;
    info.npass = np;
    if (fc && info.final_stage) {
      info.fc = S.d_fc;
      info.fc_g = b->ghost[0];
    }
    e = launch_stage<R>(h->solver, sp.recon[i], h->de != 0, S.d_sblocks + i, tiles[i],
                        S.ntiles[i], info, h->phys, 0, st);
    if (e != cudaSuccess) return cuda_fail(h, e, "stage launch");
  }
  if (h->mhd) {
    const int S1 = sp.S[sp.nstages - 1] + 1;
    e = launch_copy_faces<R>(m[0], m[1], m[2], S1, S.fface[0], S.fface[1], S.fface[2],
                             ext.f[0], ext.f[1], ext.f[2], st);
    if (e != cudaSuccess) return cuda_fail(h, e, "face copy");
  }
  return MHD_OK;
}

// The allocating block step: dt from the host (d_dt null) or from device
// memory (d_dt).
template <class R>
int block_step_t(mhdvlct_handle* h, const MhdBlockView* b, double dt, const double* d_dt,
                 const MhdFluxCorrection* fc, cudaStream_t st) {
  const int g = b->ghost[0];
  const int m[3] = {b->n[0] + 2 * g, b->n[1] + 2 * g, b->n[2] + 2 * g};
  PlainScratch<R> S;
  int rc = ensure_scratch<R>(h, m, b->dtype, S, st, b->npassive);
  if (rc) return rc;
  if (!d_dt) {
    cudaError_t e = launch_set_scalar(S.d_dt, dt, st);
    if (e != cudaSuccess) return cuda_fail(h, e, "dt upload");
    d_dt = S.d_dt;
  }
  return block_step_on<R>(h, b, S, d_dt, fc, st);
}

template <class R>
int aux_setup(mhdvlct_handle* h, const MhdBlockView* b, PlainScratch<R>& S,
              cudaStream_t st) {
  const int g = b->ghost[0];
  const int m[3] = {b->n[0] + 2 * g, b->n[1] + 2 * g, b->n[2] + 2 * g};
  int rc = ensure_scratch<R>(h, m, b->dtype, S, st, b->npassive);
  if (rc) return rc;
  AuxBlock<R> a;
  for (int k = 0; k < 3; k++) {
    a.m[k] = m[k];
    a.cw[k] = b->cell_width[k];
  }
  a.f = fieldset_of<R>(b);
  a.pressure = (R*)b->pressure;
  for (int k = 0; k < b->npassive; k++) a.pass[k] = (R*)b->passive[k];
  for (int d = 0; d < 3; d++) a.accel[d] = (R*)b->acceleration[d];
  cudaError_t e = put_bytes(S.d_aux, &a, sizeof(a), st);
  if (e != cudaSuccess) return cuda_fail(h, e, "aux upload");
  return MHD_OK;
}

// EnzoMethodMHDVlct::timestep into device memory (d_dt_out), or, with
// d_dt_out null, returned in *dt_out after a stream synchronisation.
template <class R>
int block_timestep_t(mhdvlct_handle* h, const MhdBlockView* b, double* dt_out,
                     double* d_dt_out, cudaStream_t st) {
  PlainScratch<R> S;
  int rc = aux_setup<R>(h, b, S, st);
  if (rc) return rc;
  const int g = b->ghost[0];
  const size_t M = (size_t)(b->n[0] + 2 * g) * (b->n[1] + 2 * g) * (b->n[2] + 2 * g);
  const int chunks = (int)std::min<size_t>(std::max<size_t>(1, M / 1024), 1024);
  cudaError_t e = launch_timestep<R>(h->mhd != 0, h->de != 0, S.d_aux, 1, chunks, h->phys,
                                     S.d_smax, h->params.courant, 0,
                                     d_dt_out ? d_dt_out : S.d_dtout, nullptr, st);
  if (e != cudaSuccess) return cuda_fail(h, e, "timestep launch");
  if (d_dt_out) return MHD_OK;
  e = cudaMemcpyAsync(dt_out, S.d_dtout, sizeof(double), cudaMemcpyDeviceToHost, st);
  if (e != cudaSuccess) return cuda_fail(h, e, "dt download");
  e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(h, e, "timestep");
  return MHD_OK;
}

template <class R>
int fill_ghosts_t(mhdvlct_handle* h, const MhdBlockView* b, cudaStream_t st) {
  PlainScratch<R> S;
  int rc = aux_setup<R>(h, b, S, st);
  if (rc) return rc;
  const int g = b->ghost[0];
  const int max_m = std::max(b->n[0], std::max(b->n[1], b->n[2])) + 2 * g;
  cudaError_t e = launch_refresh<R>(S.d_aux, S.d_nbr, 1, g, 64, max_m, st);
  if (e != cudaSuccess) return cuda_fail(h, e, "refresh launch");
  return MHD_OK;
}

}  // namespace

extern "C" int mhdvlct_block_step(mhdvlct_handle* h, const MhdBlockView* b,
                                  double dt, void* stream) {
  if (!h) return MHD_ERR_INVALID;
  int rc = check_view(h, b);
  if (rc) return rc;
  if (!(dt > 0) || !std::isfinite(dt)) return fail(h, MHD_ERR_INVALID, "dt must be positive and finite");
  cudaStream_t st = (cudaStream_t)stream;
  return b->dtype == MHD_DTYPE_F64 ? block_step_t<double>(h, b, dt, nullptr, nullptr, st)
                                   : block_step_t<float>(h, b, dt, nullptr, nullptr, st);
}

extern "C" int mhdvlct_block_step_fc(mhdvlct_handle* h, const MhdBlockView* b, double dt,
                                     const MhdFluxCorrection* fc, void* stream) {
  if (!h) return MHD_ERR_INVALID;
  int rc = check_view(h, b);
  if (rc) return rc;
  if (!(dt > 0) || !std::isfinite(dt)) return fail(h, MHD_ERR_INVALID, "dt must be positive and finite");
  if (!fc) return fail(h, MHD_ERR_INVALID, "null flux-correction buffers");
  // EnzoMethodMHDVlct.cpp:136-141: flux corrections only in hydro mode
  if (h->mhd)
    return fail(h, MHD_ERR_INVALID, "Flux corrections are currently only supported in hydro-mode");
  for (int d = 0; d < 3; d++)
    for (int sd = 0; sd < 2; sd++) {
      if (fc->flux[d][sd][MHD_Q_INTERNAL_ENERGY] && !h->de)
        return fail(h, MHD_ERR_INVALID, "internal_energy fluxes need dual energy");
      for (int k = b->npassive; k < 4; k++)
        if (fc->flux[d][sd][MHD_Q_PASSIVE_0 + k])
          return fail(h, MHD_ERR_INVALID, "a passive-scalar flux names a scalar the block lacks");
    }
  cudaStream_t st = (cudaStream_t)stream;
  return b->dtype == MHD_DTYPE_F64 ? block_step_t<double>(h, b, dt, nullptr, fc, st)
                                   : block_step_t<float>(h, b, dt, nullptr, fc, st);
}

extern "C" int mhdvlct_block_bfield_from_potential(mhdvlct_handle* h, const MhdBlockView* b,
                                                   const double* ax, const double* ay,
                                                   const double* az, void* stream) {
  if (!h) return MHD_ERR_INVALID;
  int rc = check_view(h, b);
  if (rc) return rc;
  if (!h->mhd) return fail(h, MHD_ERR_INVALID, "the block has no magnetic field");
  if (!ax || !ay || !az) return fail(h, MHD_ERR_INVALID, "missing vector potential");
  const int g = b->ghost[0];
  const int m[3] = {b->n[0] + 2 * g, b->n[1] + 2 * g, b->n[2] + 2 * g};
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e;
  if (b->dtype == MHD_DTYPE_F64)
    e = launch_bfield_from_potential<double>(
        m[0], m[1], m[2], ax, ay, az, b->cell_width[0], b->cell_width[1], b->cell_width[2],
        (double*)b->bfieldi[0], (double*)b->bfieldi[1], (double*)b->bfieldi[2],
        (double*)b->bfield[0], (double*)b->bfield[1], (double*)b->bfield[2], st);
  else
    e = launch_bfield_from_potential<float>(
        m[0], m[1], m[2], ax, ay, az, b->cell_width[0], b->cell_width[1], b->cell_width[2],
        (float*)b->bfieldi[0], (float*)b->bfieldi[1], (float*)b->bfieldi[2],
        (float*)b->bfield[0], (float*)b->bfield[1], (float*)b->bfield[2], st);
  return e == cudaSuccess ? MHD_OK : cuda_fail(h, e, "bfield from potential");
}

extern "C" int mhdvlct_block_timestep(mhdvlct_handle* h, const MhdBlockView* b,
                                      double* dt_out, void* stream) {
  if (!h || !dt_out) return MHD_ERR_INVALID;
  int rc = check_view(h, b);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  return b->dtype == MHD_DTYPE_F64 ? block_timestep_t<double>(h, b, dt_out, nullptr, st)
                                   : block_timestep_t<float>(h, b, dt_out, nullptr, st);
}

extern "C" int mhdvlct_block_timestep_device(mhdvlct_handle* h, const MhdBlockView* b,
                                             double* dt_dev, void* stream) {
  if (!h || !dt_dev) return MHD_ERR_INVALID;
  int rc = check_view(h, b);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  return b->dtype == MHD_DTYPE_F64 ? block_timestep_t<double>(h, b, nullptr, dt_dev, st)
                                   : block_timestep_t<float>(h, b, nullptr, dt_dev, st);
}

extern "C" int mhdvlct_block_step_device_dt(mhdvlct_handle* h, const MhdBlockView* b,
                                            const double* dt_dev, void* stream) {
  if (!h || !dt_dev) return MHD_ERR_INVALID;
  int rc = check_view(h, b);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  return b->dtype == MHD_DTYPE_F64 ? block_step_t<double>(h, b, 0.0, dt_dev, nullptr, st)
                                   : block_step_t<float>(h, b, 0.0, dt_dev, nullptr, st);
}

extern "C" int mhdvlct_dt_min_device(mhdvlct_handle* h, const double* dt_dev, int n,
                                     double* dt_min_dev, void* stream) {
  if (!h || !dt_dev || !dt_min_dev || n <= 0) return MHD_ERR_INVALID;
  cudaError_t e = launch_dt_min(dt_dev, n, dt_min_dev, (cudaStream_t)stream);
  return e == cudaSuccess ? MHD_OK : cuda_fail(h, e, "dt min");
}

extern "C" int mhdvlct_fill_ghosts_periodic(mhdvlct_handle* h, const MhdBlockView* b,
                                            void* stream) {
  if (!h) return MHD_ERR_INVALID;
  int rc = check_view(h, b);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  return b->dtype == MHD_DTYPE_F64 ? fill_ghosts_t<double>(h, b, st)
                                   : fill_ghosts_t<float>(h, b, st);
}

// ------------------------------------------------ no-allocation block step
// mhdvlct_block_step_noalloc: the plain block step with its device scratch
// in one file-scope array instead of a cudaMalloc'd buffer.  Nothing in this
// section calls cudaMalloc, cudaFree or any other allocating routine; the
// device address of the array is looked up once per device with
// cudaGetSymbolAddress and cached.
namespace {

constexpr size_t kNoAllocScratchBytes = (size_t)8 << 20;  // 8 MiB per device
constexpr int kNoAllocMaxTiles = 1024;                    // per stage
constexpr int kNoAllocMaxDevices = 64;

__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_noalloc_mu;
char* g_noalloc_base[kNoAllocMaxDevices] = {};

// Device address of the scratch array on the current device (first call per
// device resolves it; later calls read the cache).
int noalloc_base(mhdvlct_handle* h, char** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(h, e, "cudaGetDevice");
  if (dev < 0 || dev >= kNoAllocMaxDevices)
    return fail(h, MHD_ERR_INVALID, "device ordinal beyond the no-alloc scratch table");
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_base[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(h, e, "cudaGetSymbolAddress(no-alloc scratch)");
    g_noalloc_base[dev] = (char*)p;
  }
  *out = g_noalloc_base[dev];
  return MHD_OK;
}

template <class R>
int block_step_noalloc_t(mhdvlct_handle* h, const MhdBlockView* b, double dt,
                         cudaStream_t st) {
  const int g = b->ghost[0];
  const int m[3] = {b->n[0] + 2 * g, b->n[1] + 2 * g, b->n[2] + 2 * g};
  const StagePlan sp = stage_plan(h);
  const int np = b->npassive;
  // the same work decomposition as mhdvlct_block_step
  const PlainDecomp dc = plain_decomp(h, m, b->dtype);
  TileSplit ts[2] = {};
  long nt[2] = {0, 0};
  for (int i = 0; i < sp.nstages; i++) {
    ts[i] = tile_split(m, sp.S[i], i + 1 == sp.nstages, dc.tile[i], dc.tile[i], dc.zchunk[i]);
    nt[i] = ntiles_of(ts[i]);
    if (nt[i] > kNoAllocMaxTiles)
      return fail(h, MHD_ERR_INVALID,
                  "block needs more than " + std::to_string(kNoAllocMaxTiles) +
                      " tiles per stage; mhdvlct_block_step_noalloc cannot take it "
                      "(use mhdvlct_block_step)");
  }

  // carve the static array: cells, half-step scalars, stage-0 faces, final
  // faces, dt, stage descriptors, flux-output record, tiles (each region
  // 256-byte aligned)
  const size_t M = (size_t)m[0] * m[1] * m[2];
  const size_t F[3] = {(size_t)(m[0] + 1) * m[1] * m[2], (size_t)m[0] * (m[1] + 1) * m[2],
                       (size_t)m[0] * m[1] * (m[2] + 1)};
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t o = off;
    off += align_up(bytes);
    return o;
  };
  size_t o_tmp[NCELL], o_tf[3], o_ff[3], o_tp[4], o_df[3];
  for (int k = 0; k < NCELL; k++) o_tmp[k] = take(M * sizeof(R));
  for (int k = 0; k < np; k++) o_tp[k] = take(M * sizeof(R));  // half-step scalars
  for (int d = 0; d < 3 && np > 0; d++) o_df[d] = take(M * sizeof(R));  // density fluxes
  for (int d = 0; d < 3; d++) o_tf[d] = take(F[d] * sizeof(R));
  for (int d = 0; d < 3; d++) o_ff[d] = take(F[d] * sizeof(R));
  const size_t o_dt = take(sizeof(double));
  const size_t o_sb = take(2 * sizeof(StageBlock<R>));
  const size_t o_tl = take((size_t)(nt[0] + nt[1]) * sizeof(StageTile));
  if (off > kNoAllocScratchBytes)
    return fail(h, MHD_ERR_INVALID,
                "block needs " + std::to_string(off) +
                    " bytes of scratch; mhdvlct_block_step_noalloc holds at most " +
                    std::to_string(kNoAllocScratchBytes) +
                    " bytes (use mhdvlct_block_step)");

  char* base = nullptr;
  int rc = noalloc_base(h, &base);
  if (rc) return rc;
  PlainScratch<R> S{};
  for (int k = 0; k < NCELL; k++) S.tmp[k] = (R*)(base + o_tmp[k]);
  for (int k = 0; k < 4; k++) S.tpass[k] = k < np ? (R*)(base + o_tp[k]) : nullptr;
  for (int d = 0; d < 3; d++) S.dflux[d] = np > 0 ? (R*)(base + o_df[d]) : nullptr;
  for (int d = 0; d < 3; d++) {
    S.tface[d] = (R*)(base + o_tf[d]);
    S.fface[d] = (R*)(base + o_ff[d]);
  }
  S.d_dt = (double*)(base + o_dt);
  S.d_sblocks = (StageBlock<R>*)(base + o_sb);
  S.d_tiles = (StageTile*)(base + o_tl);
  S.ntiles[0] = (int)nt[0];
  S.ntiles[1] = (int)nt[1];
  S.tile[0] = dc.tile[0];
  S.tile[1] = dc.tile[1];
  // every call rewrites the dt slot, the descriptors and the tile lists (the
  // array keeps whatever the previous call left)
  cudaError_t e = launch_set_scalar(S.d_dt, dt, st);
  if (e == cudaSuccess) e = launch_make_tiles(S.d_tiles, ts[0], st);
  if (e == cudaSuccess) e = launch_make_tiles(S.d_tiles + nt[0], ts[1], st);
  if (e != cudaSuccess) return cuda_fail(h, e, "no-alloc set-up");
  return block_step_on<R>(h, b, S, S.d_dt, nullptr, st);
}

}  // namespace

extern "C" int mhdvlct_block_step_noalloc(mhdvlct_handle* h, const MhdBlockView* b,
                                          double dt, void* stream) {
  if (!h) return MHD_ERR_INVALID;
  int rc = check_view(h, b);
  if (rc) return rc;
  if (!(dt > 0) || !std::isfinite(dt)) return fail(h, MHD_ERR_INVALID, "dt must be positive and finite");
  cudaStream_t st = (cudaStream_t)stream;
  return b->dtype == MHD_DTYPE_F64 ? block_step_noalloc_t<double>(h, b, dt, st)
                                   : block_step_noalloc_t<float>(h, b, dt, st);
}
