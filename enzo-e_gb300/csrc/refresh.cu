// refresh.cu -- ghost refresh between the blocks of a mesh hierarchy:
// same-level copies, restriction into a coarser receiver and prolongation
// into a finer one, all faces of a refresh in one launch.
//
// Restates Cello's refresh of one face as FieldFace::face_to_face performs it
// (src/Cello/data_FieldFace.cpp:440-566) for a non-accumulating refresh
// created by Block::refresh_load_field_face_ (control_refresh.cpp:331-360:
// no sender ghosts, padding 0 for the "linear" prolongation):
//  - the regions come from Box (src/Cello/mesh_Box.cpp:13-234) set up by
//    FieldFace::set_box_ and box_adjust_accumulate_ (data_FieldFace.cpp:
//    982-1018);
//  - restriction is RestrictLinear::apply_ (problem_RestrictLinear.cpp:
//    53-196): the mean of the 2x2x2 fine cells, summed in the reference's
//    order and scaled by 0.125;
//  - prolongation is ProlongLinear::apply_ (problem_ProlongLinear.cpp:
//    79-310): tensor-product weights (1, 3)/4, switched to the one-sided
//    (5, -1)/4 at both ends of an axis whose coarse region has no extra
//    cells, the eight terms summed in the reference's order;
//  - fields of the "make_field_conservative" group are interpolated as
//    density-weighted values and divided by the receiver's refreshed density
//    (FieldFace::mul_by_density_ / div_by_density_, data_FieldFace.cpp:
//    863-980), only between levels.
// All arithmetic uses round-to-nearest intrinsics so that no multiply-add
// contraction changes a result: the outputs equal the reference's CPU build
// bit for bit in FP64 and FP32.
//
// Each face reads only the sender's active cells and writes only the
// receiver's ghost cells, and different senders cover disjoint parts of a
// receiver's ghost region, so all faces run concurrently in one launch.  A
// thread owns one receiver cell of one face and refreshes every field of it;
// it recomputes the receiver's density itself for the density weighting.
// The reference multiplies and divides the sender's own cells in place
// around the interpolation, which rounds them; this path leaves the sender
// untouched.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "capi_internal.h"

using namespace mhdint;

namespace {

constexpr int NSLOT = MHD_NFIELD_SLOTS;
constexpr int NCELLSLOT = MHD_FIELD_BFIELDI_X;  // cell-centred slots first
constexpr int CHUNK = 256;                      // receiver cells per CTA

// one refreshed region: a face and a set of field slots with one centering
struct RefItem {
  int type;          // -1 restrict, 0 copy, +1 prolong
  int sblk, rblk;    // block indices
  int slot0, nslot;  // field slots [slot0, slot0 + nslot)
  unsigned cons;     // density-weighted slots (between levels only)
  int is[3], ns[3];  // sender region (array indices, size)
  int id[3], nd[3];  // receiver region
  int gc[3];         // prolong: 1 when the coarse region has no extra cells
  int sm[3], rm[3];  // array extents (x, y, z) of the item's fields
  int ncell;         // nd[0] * nd[1] * nd[2]
};

struct RefChunk {
  int item, start;
};

// ------------------------------------------------------------------ host
// Regions of one face, following Box::compute_block_start, compute_region and
// get_start_stop (mesh_Box.cpp:13-225) for the two calls of face_to_face:
// (send, send, lpad) and (receive, receive, no lpad), with no sender ghosts
// and padding 0.  `type` is the receiver's level relative to the sender.
bool face_box(const int n[3], const int g[3], const int c[3], int type, const int f[3],
              const int ch[3], int is[3], int ns[3], int id[3], int nd[3]) {
  bool hit = true;
  for (int i = 0; i < 3; i++) {
    // the receiver's origin in sender cells (int, as the Box stores it)
    int bs;
    if (type == -1)
      bs = (int)(n[i] * (2.0 * f[i] - ch[i]));
    else if (type == 0)
      bs = n[i] * f[i];
    else
      bs = (int)(n[i] * (f[i] + 0.5 * ch[i]));
    // the receiver's ghosted extent in sender cells, clipped to the sender's
    // active cells
    const float ri = (float)std::pow(2.0, -1.0 * type);
    const int rs = (int)std::floor(bs - ri * g[i]);
    const int re = (int)std::ceil(bs + ri * (n[i] + g[i]));
    const int lo = std::max(0, rs), hi = std::min(n[i], re);
    // send coordinates: the region is already inside the sender's cells
    int s0 = lo, s1 = hi;
    if (!(s0 < s1)) hit = false;
    s0 += g[i];
    s1 += g[i];
    // receive coordinates: clip to the receiver's ghosted extent, map back
    const int bmin = (int)(bs + ri * (-g[i]));
    const int bmax = (int)(bs + ri * (n[i] + g[i]));
    int r0 = std::max(lo, bmin), r1 = std::min(hi, bmax);
    if (!(r0 < r1)) hit = false;
    const float r = (float)std::pow(2.0, 1.0 * type);
    r0 = (int)(g[i] + r * (r0 - bs));
    r1 = (int)(g[i] + r * (r1 - bs));
    if (c[i]) {
      if (f[i] == 0) {
        ++s1;
        ++r1;
      } else if (f[i] == -1) {
        ++s0;
        ++s1;
        ++r0;
        ++r1;
      }
    }
    is[i] = s0;
    ns[i] = s1 - s0;
    id[i] = r0;
    nd[i] = r1 - r0;
  }
  return hit;
}

bool valid_face(const MhdRefreshFace& f) {
  if (f.type < -1 || f.type > 1) return false;
  for (int a = 0; a < 3; a++) {
    if (f.face[a] < -1 || f.face[a] > 1) return false;
    if (f.child[a] < 0 || f.child[a] > 1) return false;
  }
  return f.face[0] != 0 || f.face[1] != 0 || f.face[2] != 0;
}

void slot_pointers(const MhdBlockView* b, void* p[NSLOT]) {
  p[MHD_FIELD_DENSITY] = b->density;
  for (int a = 0; a < 3; a++) {
    p[MHD_FIELD_VELOCITY_X + a] = b->velocity[a];
    p[MHD_FIELD_BFIELD_X + a] = b->bfield[a];
    p[MHD_FIELD_ACCELERATION_X + a] = b->acceleration[a];
    p[MHD_FIELD_BFIELDI_X + a] = b->bfieldi[a];
  }
  p[MHD_FIELD_TOTAL_ENERGY] = b->total_energy;
  p[MHD_FIELD_INTERNAL_ENERGY] = b->internal_energy;
  p[MHD_FIELD_PRESSURE] = b->pressure;
  for (int k = 0; k < 4; k++)
    p[MHD_FIELD_PASSIVE_0 + k] = k < b->npassive ? b->passive[k] : nullptr;
}

// ---------------------------------------------------------------- device
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double div_rn(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ float div_rn(float a, float b) { return __fdiv_rn(a, b); }

// ProlongLinear's coarse index and weights along one axis for fine index i of
// an axis of nf fine cells (problem_ProlongLinear.cpp:224-237)
template <class T>
__device__ __forceinline__ int prolong_axis(int i, int nf, int gc, T& w0, T& w1) {
  int ic = ((i + 1) >> 1) - gc;
  int w[2] = {1, 3};
  if (i == 0) ic += gc;
  if (i == nf - 1) ic -= gc;
  if (i == 0 || i == nf - 1) {
    w[0] += 4 * gc;
    w[1] -= 4 * gc;
  }
  w0 = (T)(0.25 * w[i & 1]);
  w1 = (T)(0.25 * w[~i & 1]);
  return ic;
}

template <class T>
__global__ void __launch_bounds__(CHUNK)
    refresh_faces_kernel(const RefItem* __restrict__ items, const RefChunk* __restrict__ chunks,
                         void* const* __restrict__ ptrs) {
  // the CTA's region record and both blocks' field pointers, staged once
  __shared__ RefItem it;
  __shared__ const T* src[NCELLSLOT];
  __shared__ T* dst[NCELLSLOT];
  const RefChunk ck = chunks[blockIdx.x];
  static_assert(sizeof(RefItem) % sizeof(int) == 0, "RefItem is copied as ints");
  constexpr int NW = sizeof(RefItem) / sizeof(int);
  if (threadIdx.x < NW)
    ((int*)&it)[threadIdx.x] = ((const int*)(items + ck.item))[threadIdx.x];
  __syncthreads();
  if (threadIdx.x < NCELLSLOT) {
    const int j = threadIdx.x;
    const bool in = j < it.nslot;
    src[j] = in ? (const T*)ptrs[(size_t)NSLOT * it.sblk + it.slot0 + j] : nullptr;
    dst[j] = in ? (T*)ptrs[(size_t)NSLOT * it.rblk + it.slot0 + j] : nullptr;
  }
  __syncthreads();
  const int q = ck.start + (int)threadIdx.x;
  if (q >= it.ncell) return;
  const int fx = q % it.nd[0];
  const int fy = (q / it.nd[0]) % it.nd[1];
  const int fz = q / (it.nd[0] * it.nd[1]);
  const size_t rsy = (size_t)it.rm[0], rsz = (size_t)it.rm[0] * it.rm[1];
  const size_t ssy = (size_t)it.sm[0], ssz = (size_t)it.sm[0] * it.sm[1];
  const size_t ir = (size_t)(it.id[0] + fx) + rsy * (it.id[1] + fy) + rsz * (it.id[2] + fz);
  // every value is loaded before anything is stored, so the loads of all
  // fields are in flight together (the regions read and written never
  // overlap)
  T out[NCELLSLOT];

  if (it.type == 0) {
    const size_t is = (size_t)(it.is[0] + fx) + ssy * (it.is[1] + fy) + ssz * (it.is[2] + fz);
#pragma unroll
    for (int j = 0; j < NCELLSLOT; j++)
      if (src[j]) out[j] = src[j][is];
#pragma unroll
    for (int j = 0; j < NCELLSLOT; j++)
      if (src[j]) dst[j][ir] = out[j];
    return;
  }
  size_t i0;
  T w[8];
  if (it.type == -1) {
    // the 2x2x2 fine cells under coarse cell (fx, fy, fz)
    i0 = (size_t)(it.is[0] + 2 * fx) + ssy * (it.is[1] + 2 * fy) + ssz * (it.is[2] + 2 * fz);
  } else {
    T wx[2], wy[2], wz[2];
    const int icx = prolong_axis<T>(fx, it.nd[0], it.gc[0], wx[0], wx[1]);
    const int icy = prolong_axis<T>(fy, it.nd[1], it.gc[1], wy[0], wy[1]);
    const int icz = prolong_axis<T>(fz, it.nd[2], it.gc[2], wz[0], wz[1]);
    i0 = (size_t)(it.is[0] + icx) + ssy * (it.is[1] + icy) + ssz * (it.is[2] + icz);
#pragma unroll
    for (int k = 0; k < 8; k++)
      w[k] = mul_rn(mul_rn(wx[k & 1], wy[(k >> 1) & 1]), wz[(k >> 2) & 1]);
  }
  // the eight source cells in the reference's summation order: x, y, x+y,
  // z, x+z, y+z, x+y+z
  const size_t off[8] = {0, 1, ssy, 1 + ssy, ssz, 1 + ssz, ssy + ssz, 1 + ssy + ssz};
  T rho8[8];
#pragma unroll
  for (int k = 0; k < 8; k++) rho8[k] = src[MHD_FIELD_DENSITY][i0 + off[k]];
#pragma unroll
  for (int j = 0; j < NCELLSLOT; j++) {
    if (!src[j]) continue;
    const bool cons = (it.cons >> j) & 1u;
    T sum = T(0);
#pragma unroll
    for (int k = 0; k < 8; k++) {
      const T raw = j == MHD_FIELD_DENSITY ? rho8[k] : src[j][i0 + off[k]];
      const T v = cons ? mul_rn(raw, rho8[k]) : raw;
      const T t = it.type == -1 ? v : mul_rn(w[k], v);
      sum = k == 0 ? t : add_rn(sum, t);
    }
    out[j] = it.type == -1 ? mul_rn(T(0.125), sum) : sum;
  }
  const T rho_r = out[MHD_FIELD_DENSITY];
#pragma unroll
  for (int j = 0; j < NCELLSLOT; j++) {
    if (!src[j]) continue;
    const bool cons = (it.cons >> j) & 1u;
    dst[j][ir] = cons ? div_rn(out[j], rho_r) : out[j];
  }
}

}  // namespace

namespace mhdint {

int plan_refresh(mhdvlct_handle* h, const MhdBlockView* blocks, int nblocks,
                 const MhdRefreshFace* faces, int nfaces, unsigned cons, RefreshPlan& plan) {
  const MhdBlockView& b0 = blocks[0];
  if (b0.dtype != MHD_DTYPE_F64 && b0.dtype != MHD_DTYPE_F32)
    return fail(h, MHD_ERR_INVALID, "unknown dtype");
  for (int a = 0; a < 3; a++)
    if (b0.n[a] < 1 || b0.ghost[a] < 1 || b0.n[a] + 2 * b0.ghost[a] > 4096)
      return fail(h, MHD_ERR_INVALID, "bad block extents");
  const int n[3] = {b0.n[0], b0.n[1], b0.n[2]};
  const int g[3] = {b0.ghost[0], b0.ghost[1], b0.ghost[2]};
  const int m[3] = {n[0] + 2 * g[0], n[1] + 2 * g[1], n[2] + 2 * g[2]};
  std::vector<void*>& ptrs = plan.ptrs;
  ptrs.assign((size_t)NSLOT * nblocks, nullptr);
  plan.dtype = b0.dtype;
  for (int i = 0; i < nblocks; i++) {
    const MhdBlockView& b = blocks[i];
    if (b.dtype != b0.dtype) return fail(h, MHD_ERR_INVALID, "blocks differ in dtype");
    for (int a = 0; a < 3; a++)
      if (b.n[a] != n[a] || b.ghost[a] != g[a])
        return fail(h, MHD_ERR_INVALID, "blocks differ in size or ghost depth");
    slot_pointers(&b, &ptrs[(size_t)NSLOT * i]);
    if (!ptrs[(size_t)NSLOT * i + MHD_FIELD_DENSITY])
      return fail(h, MHD_ERR_INVALID, "missing density pointer");
  }
  // the same fields on every block
  for (int i = 1; i < nblocks; i++)
    for (int s = 0; s < NSLOT; s++)
      if ((ptrs[(size_t)NSLOT * i + s] == nullptr) != (ptrs[s] == nullptr))
        return fail(h, MHD_ERR_INVALID, "blocks hold different field sets");
  for (int s = 0; s < NSLOT; s++)
    if (((cons >> s) & 1u) && (s == MHD_FIELD_DENSITY || s >= NCELLSLOT))
      return fail(h, MHD_ERR_INVALID, "only cell fields other than density can be density-weighted");
  const bool faces_b = ptrs[MHD_FIELD_BFIELDI_X] != nullptr;

  std::vector<RefItem> items;
  for (int k = 0; k < nfaces; k++) {
    const MhdRefreshFace& f = faces[k];
    if (!valid_face(f)) return fail(h, MHD_ERR_INVALID, "malformed refresh face");
    if (f.sender < 0 || f.sender >= nblocks || f.receiver < 0 || f.receiver >= nblocks)
      return fail(h, MHD_ERR_INVALID, "refresh face names a block out of range");
    if (f.type != 0 && faces_b)
      return fail(h, MHD_ERR_INVALID,
                  "face-centred B cannot be restricted or prolonged (no such operator)");
    for (int pass = 0; pass < (f.type == 0 && faces_b ? 4 : 1); pass++) {
      // pass 0: the cell fields; pass 1..3: bfieldi along axis pass-1
      int c[3] = {0, 0, 0};
      int ext[3] = {m[0], m[1], m[2]};
      if (pass > 0) {
        c[pass - 1] = 1;
        ext[pass - 1] += 1;
      }
      RefItem it{};
      it.type = f.type;
      it.sblk = f.sender;
      it.rblk = f.receiver;
      it.slot0 = pass == 0 ? 0 : MHD_FIELD_BFIELDI_X + pass - 1;
      it.nslot = pass == 0 ? NCELLSLOT : 1;
      it.cons = f.type != 0 ? cons : 0u;
      if (!face_box(n, g, c, f.type, f.face, f.child, it.is, it.ns, it.id, it.nd)) continue;
      long ncell = 1;
      for (int a = 0; a < 3; a++) {
        it.sm[a] = it.rm[a] = ext[a];
        if (it.ns[a] <= 0 || it.nd[a] <= 0) ncell = 0;
        ncell *= std::max(it.nd[a], 0);
      }
      if (ncell == 0) continue;
      // the reference's consistency checks, and every access in bounds
      for (int a = 0; a < 3; a++) {
        int lo, hi;  // sender cells read along this axis
        if (f.type == 0) {
          if (it.nd[a] != it.ns[a])
            return fail(h, MHD_ERR_INVALID, "copy regions differ in size");
          lo = it.is[a];
          hi = it.is[a] + it.ns[a];
        } else if (f.type == -1) {
          if (2 * it.nd[a] != it.ns[a])
            return fail(h, MHD_ERR_INVALID,
                        "restriction needs a fine region twice the coarse one (even ghost depth)");
          lo = it.is[a];
          hi = it.is[a] + 2 * it.nd[a];
        } else {
          if (it.nd[a] == 2 * it.ns[a])
            it.gc[a] = 1;
          else if (it.nd[a] == 2 * (it.ns[a] - 2))
            it.gc[a] = 0;
          else
            return fail(h, MHD_ERR_INVALID,
                        "fine region must be 2 times the coarse one (even ghost depth)");
          // coarse indices the weights touch: ic and ic+1 over the axis
          lo = 1 << 30;
          hi = -(1 << 30);
          for (int i = 0; i < it.nd[a]; i++) {
            int ic = ((i + 1) >> 1) - it.gc[a];
            if (i == 0) ic += it.gc[a];
            if (i == it.nd[a] - 1) ic -= it.gc[a];
            lo = std::min(lo, it.is[a] + ic);
            hi = std::max(hi, it.is[a] + ic + 2);
          }
        }
        if (lo < 0 || hi > it.sm[a] || it.id[a] < 0 || it.id[a] + it.nd[a] > it.rm[a])
          return fail(h, MHD_ERR_INVALID, "refresh region outside the block arrays");
      }
      it.ncell = (int)ncell;
      items.push_back(it);
    }
  }
  std::vector<RefChunk> chunks;
  for (int k = 0; k < (int)items.size(); k++)
    for (int s = 0; s < items[k].ncell; s += CHUNK) chunks.push_back({k, s});

  plan.items.assign((const char*)items.data(), (const char*)(items.data() + items.size()));
  plan.chunks.assign((const char*)chunks.data(), (const char*)(chunks.data() + chunks.size()));
  plan.nchunks = (int)chunks.size();
  return MHD_OK;
}

cudaError_t launch_refresh_faces(int dtype, const void* d_items, const void* d_chunks,
                                 int nchunks, void* const* d_ptrs, cudaStream_t st) {
  if (nchunks <= 0) return cudaSuccess;
  if (dtype == MHD_DTYPE_F64)
    refresh_faces_kernel<double><<<(unsigned)nchunks, CHUNK, 0, st>>>(
        (const RefItem*)d_items, (const RefChunk*)d_chunks, d_ptrs);
  else
    refresh_faces_kernel<float><<<(unsigned)nchunks, CHUNK, 0, st>>>(
        (const RefItem*)d_items, (const RefChunk*)d_chunks, d_ptrs);
  return cudaGetLastError();
}

}  // namespace mhdint

namespace {

int refresh_t(mhdvlct_handle* h, const MhdBlockView* blocks, int nblocks,
              const MhdRefreshFace* faces, int nfaces, unsigned cons, cudaStream_t st) {
  RefreshPlan plan;
  int rc = plan_refresh(h, blocks, nblocks, faces, nfaces, cons, plan);
  if (rc != MHD_OK || plan.nchunks == 0) return rc;
  // one upload: pointer table, items, chunks
  const size_t b_ptr = plan.ptrs.size() * sizeof(void*);
  const size_t o_items = (b_ptr + 255) / 256 * 256;
  const size_t b_items = plan.items.size();
  const size_t o_chunks = (o_items + b_items + 255) / 256 * 256;
  const size_t total = o_chunks + plan.chunks.size();
  // the previous launch must be done with the tables before they are rewritten
  cudaError_t e = cudaSuccess;
  if (h->rf_done && (e = cudaEventSynchronize(h->rf_done)) != cudaSuccess)
    return fail(h, MHD_ERR_CUDA, std::string("refresh: ") + cudaGetErrorString(e));
  if (!h->rf_done && (e = cudaEventCreateWithFlags(&h->rf_done, cudaEventDisableTiming)) !=
                         cudaSuccess)
    return fail(h, MHD_ERR_CUDA, std::string("refresh event: ") + cudaGetErrorString(e));
  if (h->rf_bytes < total) {
    if (h->rf_dev) cudaFree(h->rf_dev);
    h->rf_dev = nullptr;
    h->rf_bytes = 0;
    if (cudaMalloc(&h->rf_dev, total) != cudaSuccess)
      return fail(h, MHD_ERR_NOMEM, "refresh tables");
    h->rf_bytes = total;
  }
  h->rf_host.assign(total, 0);
  memcpy(h->rf_host.data(), plan.ptrs.data(), b_ptr);
  memcpy(h->rf_host.data() + o_items, plan.items.data(), b_items);
  memcpy(h->rf_host.data() + o_chunks, plan.chunks.data(), plan.chunks.size());
  e = cudaMemcpyAsync(h->rf_dev, h->rf_host.data(), total, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess)
    return fail(h, MHD_ERR_CUDA, std::string("refresh upload: ") + cudaGetErrorString(e));
  const char* d = (const char*)h->rf_dev;
  e = launch_refresh_faces(plan.dtype, d + o_items, d + o_chunks, plan.nchunks,
                           (void* const*)d, st);
  if (e == cudaSuccess) e = cudaEventRecord(h->rf_done, st);
  if (e != cudaSuccess)
    return fail(h, MHD_ERR_CUDA, std::string("refresh launch: ") + cudaGetErrorString(e));
  return MHD_OK;
}

}  // namespace

extern "C" int mhdvlct_refresh_faces(mhdvlct_handle* h, const MhdBlockView* blocks,
                                     int nblocks, const MhdRefreshFace* faces, int nfaces,
                                     unsigned conservative, void* stream) {
  if (!h) return MHD_ERR_INVALID;
  if (!blocks || nblocks <= 0 || nfaces < 0 || (nfaces > 0 && !faces))
    return fail(h, MHD_ERR_INVALID, "bad refresh arguments");
  if (blocks[0].dtype != MHD_DTYPE_F64 && blocks[0].dtype != MHD_DTYPE_F32)
    return fail(h, MHD_ERR_INVALID, "unknown dtype");
  for (int a = 0; a < 3; a++)
    if (blocks[0].n[a] < 1 || blocks[0].ghost[a] < 1 ||
        blocks[0].n[a] + 2 * blocks[0].ghost[a] > 4096)
      return fail(h, MHD_ERR_INVALID, "bad block extents");
  return refresh_t(h, blocks, nblocks, faces, nfaces, conservative, (cudaStream_t)stream);
}

extern "C" int mhdvlct_refresh_face_box(const int n[3], const int ghost[3],
                                        const int centering[3], int type, const int face[3],
                                        const int child[3], int send_start[3],
                                        int send_size[3], int recv_start[3],
                                        int recv_size[3]) {
  if (!n || !ghost || !centering || !face || !child || !send_start || !send_size ||
      !recv_start || !recv_size)
    return -1;
  MhdRefreshFace f{};
  f.type = type;
  for (int a = 0; a < 3; a++) {
    f.face[a] = face[a];
    f.child[a] = child[a];
    if (n[a] < 1 || ghost[a] < 0 || centering[a] < 0 || centering[a] > 1) return -1;
  }
  if (!valid_face(f)) return -1;
  const bool hit = face_box(n, ghost, centering, type, face, child, send_start, send_size,
                            recv_start, recv_size);
  for (int a = 0; a < 3; a++)
    if (send_size[a] <= 0 || recv_size[a] <= 0) return 0;
  return hit ? 1 : 0;
}
