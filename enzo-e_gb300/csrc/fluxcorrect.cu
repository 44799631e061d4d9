// fluxcorrect.cu -- flux correction at coarse-fine faces (Cello's
// "flux_correct" Method) for blocks whose boundary fluxes the step stored.
//
// Restates, per corrected cell of a coarse block:
//  - FaceFluxes::coarsen (src/Cello/data_FaceFluxes.cpp:128-252) of each
//    finer neighbour's stored fluxes: every fine face adds 0.25 * 0.125 times
//    its flux four times into the coarse face that covers it, fine faces
//    visited inner index fastest; in an FP32 build each add is done in double
//    and rounded to float, as the reference's mixed-type expression does;
//  - FluxData::sum_neighbor_fluxes (data_FluxData.hpp:136-145): the
//    coarsened arrays summed into a zeroed neighbour-flux array;
//  - MethodFluxCorrect::flux_correct_ and its helpers
//    (src/Cello/problem_MethodFluxCorrect.cpp:293-558): on every face whose
//    neighbour is finer, the boundary layer of active cells gets
//    (2 face - 1) (own flux - neighbour flux), faces in (axis, face) order;
//    density first; a "make_field_conservative" field is corrected as
//    old density times its value and divided by the corrected density.
// One thread owns one boundary cell: the first corrected face (in that
// order) containing the cell claims it and applies every correction of the
// cell, so cells on edges and corners are never updated by two threads.
// Arithmetic uses round-to-nearest intrinsics (no contraction): FP64 and
// FP32 results equal the reference's bit for bit.
#include <cuda_runtime.h>

#include <cstring>
#include <string>
#include <vector>

#include "capi_internal.h"

using namespace mhdint;

namespace {

constexpr int NQ = MHD_FC_NQ;  // MHD_Q_*: six hydro quantities, four passive scalars
constexpr int FC_CHUNK = 256;

// one corrected face of a coarse block
struct FcFace {
  int blk;             // the coarse block
  int axis, face;      // the coarse block's face (face 0 = low)
  int child[2][2];     // [outer][inner] transverse child -> finer block index
  int faces_of_blk[6]; // the block's corrected faces (index or -1), (axis, face) order
  int ncell;           // cells of the layer: n_inner * n_outer
};

struct FcChunk {
  int face, start;
};

// per-block device pointers: the corrected fields and the stored fluxes
struct FcBlockPtrs {
  void* field[NQ];          // density, velocity_x/y/z, total_energy, internal_energy,
                            // passive scalars 0-3 (conserved form)
  void* flux[3][2][NQ];
};

struct FcParams {
  int n[3], m[3], g;
  unsigned qmask;  // quantities stored
  unsigned cons;   // density-weighted quantities (MHD_Q_* bits)
};

__device__ __forceinline__ double fadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double fsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double fmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double fdiv(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }

// one add of FaceFluxes::coarsen: c += 0.25 * dArea * f in double, then
// stored in the field type
__device__ __forceinline__ double coarsen_add(double c, double f) {
  return __dadd_rn(c, __dmul_rn(0.03125, f));
}
__device__ __forceinline__ float coarsen_add(float c, float f) {
  return __double2float_rn(__dadd_rn((double)c, __dmul_rn(0.03125, (double)f)));
}

// transverse axes of a face: inner (fastest in the face arrays) and outer
__device__ __forceinline__ void transverse(int axis, int& a_in, int& a_out) {
  a_in = axis == 0 ? 1 : 0;
  a_out = axis == 2 ? 1 : 2;
}

template <class T>
__global__ void __launch_bounds__(FC_CHUNK)
    flux_correct_kernel(const FcFace* __restrict__ faces, const FcChunk* __restrict__ chunks,
                        const FcBlockPtrs* __restrict__ bp, FcParams P) {
  const FcChunk ck = chunks[blockIdx.x];
  const FcFace& F = faces[ck.face];
  const int q = ck.start + (int)threadIdx.x;
  if (q >= F.ncell) return;
  int a_in, a_out;
  transverse(F.axis, a_in, a_out);
  int c[3];  // active coordinates of the cell
  c[a_in] = q % P.n[a_in];
  c[a_out] = q / P.n[a_in];
  c[F.axis] = F.face == 0 ? 0 : P.n[F.axis] - 1;
  const int self = F.axis * 2 + F.face;
  // the first corrected face containing the cell owns it
  for (int k = 0; k < self; k++) {
    if (F.faces_of_blk[k] < 0) continue;
    const int ax = k >> 1, fc = k & 1;
    if (c[ax] == (fc == 0 ? 0 : P.n[ax] - 1)) return;
  }
  const FcBlockPtrs& B = bp[F.blk];
  const size_t cell = (size_t)(c[0] + P.g) +
                      (size_t)P.m[0] * ((size_t)(c[1] + P.g) + (size_t)P.m[1] * (c[2] + P.g));
  // the corrected faces containing the cell, in (axis, face) order
  int list[3], nl = 0;
  for (int k = 0; k < 6; k++) {
    if (F.faces_of_blk[k] < 0) continue;
    const int ax = k >> 1, fc = k & 1;
    if (c[ax] == (fc == 0 ? 0 : P.n[ax] - 1)) list[nl++] = F.faces_of_blk[k];
  }
  // (2 face - 1) (own flux - neighbour flux) of quantity qq through face fi
  auto correction = [&](int fi, int qq) -> T {
    const FcFace& G = faces[fi];
    int gi, go;
    transverse(G.axis, gi, go);
    const int ni = P.n[gi], no = P.n[go];
    const int j = c[gi], k = c[go];
    const T fb = ((const T*)B.flux[G.axis][G.face][qq])[(size_t)k * ni + j];
    const int hi = ni / 2, ho = no / 2;
    const int cj = j / hi, ckk = k / ho;
    const T* fine = (const T*)bp[G.child[ckk][cj]].flux[G.axis][1 - G.face][qq];
    const int j0 = 2 * (j - cj * hi), k0 = 2 * (k - ckk * ho);
    T s = T(0);
#pragma unroll
    for (int dk = 0; dk < 2; dk++)
#pragma unroll
      for (int dj = 0; dj < 2; dj++) {
        const T f = fine[(size_t)(k0 + dk) * ni + (j0 + dj)];
#pragma unroll
        for (int r = 0; r < 4; r++) s = coarsen_add(s, f);
      }
    const T fn = fadd(T(0), s);  // the zeroed neighbour-flux array plus it
    const T d = fsub(fb, fn);
    return G.face == 1 ? d : fmul(T(-1), d);
  };
  T* rho = (T*)B.field[MHD_Q_DENSITY];
  const T rho_old = rho[cell];
  T rho_new = rho_old;
  if (P.qmask & 1u) {
    for (int l = 0; l < nl; l++) rho_new = fadd(rho_new, correction(list[l], MHD_Q_DENSITY));
    rho[cell] = rho_new;
  }
  for (int qq = 1; qq < NQ; qq++) {
    if (!((P.qmask >> qq) & 1u)) continue;
    T* u = (T*)B.field[qq];
    if ((P.cons >> qq) & 1u) {
      T t = fmul(rho_old, u[cell]);
      for (int l = 0; l < nl; l++) t = fadd(t, correction(list[l], qq));
      u[cell] = fdiv(t, rho_new);
    } else {
      T v = u[cell];
      for (int l = 0; l < nl; l++) v = fadd(v, correction(list[l], qq));
      u[cell] = v;
    }
  }
}

}  // namespace

namespace mhdint {

int plan_flux_correct(mhdvlct_handle* h, const MhdBlockView* blocks, int nblocks,
                      const MhdFluxCorrection* fluxes, const MhdRefreshFace* faces,
                      int nfaces, unsigned conservative, FluxCorrectPlan& plan) {
  plan = FluxCorrectPlan();
  if (!blocks || !fluxes || nblocks <= 0 || nfaces < 0 || (nfaces > 0 && !faces))
    return fail(h, MHD_ERR_INVALID, "bad flux-correction arguments");
  const MhdBlockView& b0 = blocks[0];
  if (b0.dtype != MHD_DTYPE_F64 && b0.dtype != MHD_DTYPE_F32)
    return fail(h, MHD_ERR_INVALID, "unknown dtype");
  FcParams P{};
  P.g = b0.ghost[0];
  for (int a = 0; a < 3; a++) {
    P.n[a] = b0.n[a];
    P.m[a] = b0.n[a] + 2 * b0.ghost[a];
    if (b0.ghost[a] != P.g || P.n[a] < 2 || (P.n[a] & 1) || P.m[a] > 4096)
      return fail(h, MHD_ERR_INVALID, "block extents must be even and equal ghost depths");
  }
  // the stored quantities: the same on every block and face
  unsigned qmask = 0;
  for (int q = 0; q < NQ; q++)
    if (fluxes[0].flux[0][0][q]) qmask |= 1u << q;
  std::vector<FcBlockPtrs> bp(nblocks);
  for (int i = 0; i < nblocks; i++) {
    const MhdBlockView& b = blocks[i];
    if (b.dtype != b0.dtype) return fail(h, MHD_ERR_INVALID, "blocks differ in dtype");
    for (int a = 0; a < 3; a++)
      if (b.n[a] != b0.n[a] || b.ghost[a] != b0.ghost[a])
        return fail(h, MHD_ERR_INVALID, "blocks differ in size or ghost depth");
    FcBlockPtrs& p = bp[i];
    p.field[MHD_Q_DENSITY] = b.density;
    for (int a = 0; a < 3; a++) p.field[MHD_Q_VELOCITY_X + a] = b.velocity[a];
    p.field[MHD_Q_TOTAL_ENERGY] = b.total_energy;
    p.field[MHD_Q_INTERNAL_ENERGY] = b.internal_energy;
    for (int k = 0; k < 4; k++)
      p.field[MHD_Q_PASSIVE_0 + k] = k < b.npassive ? b.passive[k] : nullptr;
    for (int a = 0; a < 3; a++)
      for (int s = 0; s < 2; s++)
        for (int q = 0; q < NQ; q++) {
          p.flux[a][s][q] = fluxes[i].flux[a][s][q];
          if ((p.flux[a][s][q] != nullptr) != (((qmask >> q) & 1u) != 0))
            return fail(h, MHD_ERR_INVALID, "every block and face must store the same fluxes");
        }
    for (int q = 0; q < NQ; q++)
      if (((qmask >> q) & 1u) && !p.field[q])
        return fail(h, MHD_ERR_INVALID, "a corrected field is missing from a block view");
  }
  if (((qmask >> 1) & 7u) != 0 && ((qmask >> 1) & 7u) != 7u)
    return fail(h, MHD_ERR_INVALID, "store all three momentum fluxes or none");
  // the conservative mask in MHD_Q_* bits (field slots 1..5 are the same;
  // the passive scalars' field slots start at MHD_FIELD_PASSIVE_0).  Without
  // a stored density flux a density-weighted field is divided by the
  // uncorrected density, as the reference does.
  P.qmask = qmask;
  P.cons = 0;
  for (int q = 1; q < MHD_Q_PASSIVE_0; q++)
    if ((conservative >> q) & 1u) P.cons |= 1u << q;
  for (int k = 0; k < 4; k++)
    if ((conservative >> (MHD_FIELD_PASSIVE_0 + k)) & 1u) P.cons |= 1u << (MHD_Q_PASSIVE_0 + k);
  // corrected faces: (coarse block, axis, face) <- four finer children
  std::vector<int> index((size_t)nblocks * 6, -1);
  std::vector<FcFace> fl;
  for (int k = 0; k < nfaces; k++) {
    const MhdRefreshFace& f = faces[k];
    if (f.type != MHD_REFRESH_COARSE) continue;
    const int nz = (f.face[0] != 0) + (f.face[1] != 0) + (f.face[2] != 0);
    if (nz != 1) continue;  // fluxes live on axis faces only
    if (f.sender < 0 || f.sender >= nblocks || f.receiver < 0 || f.receiver >= nblocks)
      return fail(h, MHD_ERR_INVALID, "refresh face names a block out of range");
    const int axis = f.face[0] ? 0 : (f.face[1] ? 1 : 2);
    if (f.face[axis] != 1 && f.face[axis] != -1)
      return fail(h, MHD_ERR_INVALID, "malformed refresh face");
    const int face = f.face[axis] == 1 ? 0 : 1;  // the coarse block's side
    const int a_in = axis == 0 ? 1 : 0, a_out = axis == 2 ? 1 : 2;
    const int ci = f.child[a_in], co = f.child[a_out];
    if (ci < 0 || ci > 1 || co < 0 || co > 1)
      return fail(h, MHD_ERR_INVALID, "malformed child index");
    int& slot = index[(size_t)f.receiver * 6 + axis * 2 + face];
    if (slot < 0) {
      slot = (int)fl.size();
      FcFace nf{};
      nf.blk = f.receiver;
      nf.axis = axis;
      nf.face = face;
      for (int u = 0; u < 2; u++)
        for (int v = 0; v < 2; v++) nf.child[u][v] = -1;
      nf.ncell = P.n[a_in] * P.n[a_out];
      fl.push_back(nf);
    }
    if (fl[slot].child[co][ci] >= 0)
      return fail(h, MHD_ERR_INVALID, "two finer neighbours claim the same quarter face");
    fl[slot].child[co][ci] = f.sender;
  }
  if (fl.empty() || qmask == 0) return MHD_OK;
  for (auto& f : fl) {
    for (int u = 0; u < 2; u++)
      for (int v = 0; v < 2; v++)
        if (f.child[u][v] < 0)
          return fail(h, MHD_ERR_INVALID, "a coarse face lacks one of its four finer neighbours");
    for (int k = 0; k < 6; k++) f.faces_of_blk[k] = index[(size_t)f.blk * 6 + k];
  }
  std::vector<FcChunk> chunks;
  for (int k = 0; k < (int)fl.size(); k++)
    for (int s = 0; s < fl[k].ncell; s += FC_CHUNK) chunks.push_back({k, s});

  const size_t b_faces = fl.size() * sizeof(FcFace);
  plan.o_chunks = (b_faces + 255) / 256 * 256;
  plan.o_blocks = (plan.o_chunks + chunks.size() * sizeof(FcChunk) + 255) / 256 * 256;
  plan.blob.assign(plan.o_blocks + bp.size() * sizeof(FcBlockPtrs), 0);
  memcpy(plan.blob.data(), fl.data(), b_faces);
  memcpy(plan.blob.data() + plan.o_chunks, chunks.data(), chunks.size() * sizeof(FcChunk));
  memcpy(plan.blob.data() + plan.o_blocks, bp.data(), bp.size() * sizeof(FcBlockPtrs));
  plan.nchunks = (int)chunks.size();
  plan.dtype = b0.dtype;
  static_assert(sizeof(FcParams) == sizeof(plan.params), "kernel parameters");
  memcpy(plan.params, &P, sizeof(P));
  return MHD_OK;
}

cudaError_t launch_flux_correct(const FluxCorrectPlan& plan, const void* d_blob,
                                cudaStream_t st) {
  if (plan.nchunks <= 0) return cudaSuccess;
  FcParams P;
  memcpy(&P, plan.params, sizeof(P));
  const char* dc = (const char*)d_blob;
  if (plan.dtype == MHD_DTYPE_F64)
    flux_correct_kernel<double><<<(unsigned)plan.nchunks, FC_CHUNK, 0, st>>>(
        (const FcFace*)dc, (const FcChunk*)(dc + plan.o_chunks),
        (const FcBlockPtrs*)(dc + plan.o_blocks), P);
  else
    flux_correct_kernel<float><<<(unsigned)plan.nchunks, FC_CHUNK, 0, st>>>(
        (const FcFace*)dc, (const FcChunk*)(dc + plan.o_chunks),
        (const FcBlockPtrs*)(dc + plan.o_blocks), P);
  return cudaGetLastError();
}

}  // namespace mhdint

extern "C" int mhdvlct_flux_correct(mhdvlct_handle* h, const MhdBlockView* blocks, int nblocks,
                                    const MhdFluxCorrection* fluxes,
                                    const MhdRefreshFace* faces, int nfaces,
                                    unsigned conservative, void* stream) {
  if (!h) return MHD_ERR_INVALID;
  FluxCorrectPlan plan;
  int rc = plan_flux_correct(h, blocks, nblocks, fluxes, faces, nfaces, conservative, plan);
  if (rc != MHD_OK || plan.nchunks == 0) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  void* d = nullptr;
  // a one-off plan per call: allocate, upload, launch, free after the stream
  // has consumed it
  cudaError_t e = cudaMallocAsync(&d, plan.blob.size(), st);
  if (e != cudaSuccess) return fail(h, MHD_ERR_NOMEM, "flux-correction tables");
  e = cudaMemcpyAsync(d, plan.blob.data(), plan.blob.size(), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = launch_flux_correct(plan, d, st);
  // the host staging buffer is consumed once the copy has run
  cudaError_t e2 = cudaStreamSynchronize(st);
  cudaFreeAsync(d, st);
  if (e == cudaSuccess) e = e2;
  if (e != cudaSuccess)
    return fail(h, MHD_ERR_CUDA, std::string("flux correction: ") + cudaGetErrorString(e));
  return MHD_OK;
}
