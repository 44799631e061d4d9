/*
 * refresh_oracle.cpp -- TEST INFRASTRUCTURE ONLY.
 *
 * A CPU restatement of Cello's ghost refresh of one face between blocks of
 * the same or adjacent refinement levels, as FieldFace::face_to_face runs it
 * (src/Cello/data_FieldFace.cpp:440-566) for a non-accumulating refresh made
 * by Block::refresh_load_field_face_ (src/Cello/control_refresh.cpp:331-360)
 * with the "linear" prolongation and restriction.  Regions follow Box
 * (src/Cello/mesh_Box.cpp:13-234); the operators follow ProlongLinear::apply_
 * (problem_ProlongLinear.cpp:79-310) and RestrictLinear::apply_
 * (problem_RestrictLinear.cpp:53-196) in the same operation order, compiled
 * with -ffp-contract=off.  Density-weighted fields use the sender's density
 * on the fly instead of scaling the sender in place, and leave the sender
 * unchanged.  No code here is shared with the CUDA product.
 */
#include <algorithm>
#include <cmath>
#include <cstddef>

namespace {

const int NSLOT = 20;  // 17 cell-centred field slots, then bfieldi_x/y/z
const int NCELL = 17;

// The Box of one face (mesh_Box.cpp), for a sender with no send ghosts and no
// padding; level = the receiver's level relative to the sender's.
struct FaceRegion {
  int n[3], g[3], c[3], level, face[3], child[3];
  int start[3];           // Box::block_start_[receive]
  int lo[3], hi[3];       // Box::region_start_ / region_stop_

  void block_start() {  // Box::compute_block_start (mesh_Box.cpp:13-34)
    for (int i = 0; i < 3; i++) {
      if (level == -1)
        start[i] = n[i] * (2.0 * face[i] - child[i]);
      else if (level == 0)
        start[i] = n[i] * face[i];
      else
        start[i] = n[i] * (face[i] + 0.5 * child[i]);
    }
  }
  void region() {  // Box::compute_region (mesh_Box.cpp:38-57)
    const float ri = std::pow(2.0, -1.0 * level);
    for (int i = 0; i < 3; i++) {
      const int a = int(std::floor(start[i] - ri * g[i]));
      const int b = int(std::ceil(start[i] + ri * (n[i] + g[i])));
      lo[i] = std::max(0, a);
      hi[i] = std::min(n[i], b);
    }
  }
  // Box::get_start_stop (mesh_Box.cpp:76-207) and get_start_size
  void send(int i0[3], int n0[3]) const {
    for (int i = 0; i < 3; i++) {
      int a = std::max(lo[i], 0), b = std::min(hi[i], n[i]);
      a += g[i];
      b += g[i];
      centre(i, a, b);
      i0[i] = a;
      n0[i] = b - a;
    }
  }
  void receive(int i0[3], int n0[3]) const {
    const float r = std::pow(2.0, -1.0 * level);
    const float rr = std::pow(2.0, 1.0 * level);
    for (int i = 0; i < 3; i++) {
      const int bmin = start[i] + r * (-g[i]);
      const int bmax = start[i] + r * (n[i] + g[i]);
      int a = std::max(lo[i], bmin), b = std::min(hi[i], bmax);
      a = g[i] + rr * (a - start[i]);
      b = g[i] + rr * (b - start[i]);
      centre(i, a, b);
      i0[i] = a;
      n0[i] = b - a;
    }
  }
  void centre(int i, int& a, int& b) const {
    if (!c[i]) return;
    if (face[i] == 0) {
      ++b;
    } else if (face[i] == -1) {
      ++a;
      ++b;
    }
  }
};

FaceRegion make_region(const int n[3], const int g[3], const int c[3], int level,
                       const int face[3], const int child[3]) {
  FaceRegion fr;
  for (int i = 0; i < 3; i++) {
    fr.n[i] = n[i];
    fr.g[i] = g[i];
    fr.c[i] = c[i];
    fr.face[i] = face[i];
    fr.child[i] = child[i];
  }
  fr.level = level;
  fr.block_start();
  fr.region();
  return fr;
}

// value of slot `s` at flat index i of the sender, density-weighted if asked
template <class T>
inline T src_value(T* const* sf, int s, size_t i, bool weighted) {
  return weighted ? sf[s][i] * sf[0][i] : sf[s][i];
}

template <class T>
int refresh(int nblocks, const int n[3], const int g[3], void* const* fields,
            const int* faces, int nfaces, unsigned cons) {
  for (int k = 0; k < nfaces; k++) {
    const int* fc = faces + 9 * k;
    const int s = fc[0], r = fc[1], level = fc[2];
    if (s < 0 || s >= nblocks || r < 0 || r >= nblocks || level < -1 || level > 1) return 1;
    T* const* sf = (T* const*)(fields + (size_t)NSLOT * s);
    T* const* rf = (T* const*)(fields + (size_t)NSLOT * r);
    for (int slot = 0; slot < NSLOT; slot++) {
      if (!sf[slot]) continue;
      int c[3] = {0, 0, 0};
      if (slot >= NCELL) {
        if (level != 0) return 2;
        c[slot - NCELL] = 1;
      }
      const int m[3] = {n[0] + 2 * g[0] + c[0], n[1] + 2 * g[1] + c[1], n[2] + 2 * g[2] + c[2]};
      const FaceRegion fr = make_region(n, g, c, level, fc + 3, fc + 6);
      int is[3], ns[3], id[3], nd[3];
      fr.send(is, ns);
      fr.receive(id, nd);
      const size_t sy = m[0], sz = (size_t)m[0] * m[1];
      const bool weighted = level != 0 && ((cons >> slot) & 1u);
      T* dst = rf[slot];
      if (level == 0) {  // FieldFace::copy_ (data_FieldFace.cpp:806-841)
        for (int z = 0; z < ns[2]; z++)
          for (int y = 0; y < ns[1]; y++)
            for (int x = 0; x < ns[0]; x++)
              dst[(id[0] + x) + sy * (id[1] + y) + sz * (id[2] + z)] =
                  sf[slot][(is[0] + x) + sy * (is[1] + y) + sz * (is[2] + z)];
        continue;
      }
      if (level == -1) {  // RestrictLinear::apply_, rank 3 (problem_RestrictLinear.cpp:140-165)
        for (int z = 0; z < nd[2]; z++)
          for (int y = 0; y < nd[1]; y++)
            for (int x = 0; x < nd[0]; x++) {
              const size_t f = (is[0] + 2 * x) + sy * (is[1] + 2 * y) + sz * (is[2] + 2 * z);
              const T sum = src_value(sf, slot, f, weighted) +
                            src_value(sf, slot, f + 1, weighted) +
                            src_value(sf, slot, f + sy, weighted) +
                            src_value(sf, slot, f + 1 + sy, weighted) +
                            src_value(sf, slot, f + sz, weighted) +
                            src_value(sf, slot, f + 1 + sz, weighted) +
                            src_value(sf, slot, f + sy + sz, weighted) +
                            src_value(sf, slot, f + 1 + sy + sz, weighted);
              dst[(id[0] + x) + sy * (id[1] + y) + sz * (id[2] + z)] = 0.125 * sum;
            }
      } else {  // ProlongLinear::apply_, rank 3 (problem_ProlongLinear.cpp:214-298)
        int gc[3];
        for (int i = 0; i < 3; i++) {
          if (nd[i] == 2 * ns[i])
            gc[i] = 1;
          else if (nd[i] == 2 * (ns[i] - 2))
            gc[i] = 0;
          else
            return 3;  // the reference asserts here
        }
        auto axis = [](int i, int nf, int gcc, T& w0, T& w1) {
          int ic = ((i + 1) >> 1) - gcc;
          int w[2] = {1, 3};
          if (i == 0) ic += gcc;
          if (i == nf - 1) ic -= gcc;
          if (i == 0 || i == nf - 1) {
            w[0] += 4 * gcc;
            w[1] -= 4 * gcc;
          }
          w0 = 0.25 * w[i & 1];
          w1 = 0.25 * w[~i & 1];
          return ic;
        };
        for (int z = 0; z < nd[2]; z++) {
          T z0, z1;
          const int cz = axis(z, nd[2], gc[2], z0, z1);
          for (int y = 0; y < nd[1]; y++) {
            T y0, y1;
            const int cy = axis(y, nd[1], gc[1], y0, y1);
            for (int x = 0; x < nd[0]; x++) {
              T x0, x1;
              const int cx = axis(x, nd[0], gc[0], x0, x1);
              const size_t ci = (is[0] + cx) + sy * (is[1] + cy) + sz * (is[2] + cz);
              const T v = x0 * y0 * z0 * src_value(sf, slot, ci, weighted) +
                          x1 * y0 * z0 * src_value(sf, slot, ci + 1, weighted) +
                          x0 * y1 * z0 * src_value(sf, slot, ci + sy, weighted) +
                          x1 * y1 * z0 * src_value(sf, slot, ci + 1 + sy, weighted) +
                          x0 * y0 * z1 * src_value(sf, slot, ci + sz, weighted) +
                          x1 * y0 * z1 * src_value(sf, slot, ci + 1 + sz, weighted) +
                          x0 * y1 * z1 * src_value(sf, slot, ci + sy + sz, weighted) +
                          x1 * y1 * z1 * src_value(sf, slot, ci + 1 + sy + sz, weighted);
              dst[(id[0] + x) + sy * (id[1] + y) + sz * (id[2] + z)] = v;
            }
          }
        }
      }
      if (weighted)  // FieldFace::div_by_density_ on the receiver's region
        for (int z = 0; z < nd[2]; z++)
          for (int y = 0; y < nd[1]; y++)
            for (int x = 0; x < nd[0]; x++) {
              const size_t i = (id[0] + x) + sy * (id[1] + y) + sz * (id[2] + z);
              dst[i] /= rf[0][i];
            }
    }
  }
  return 0;
}

}  // namespace

extern "C" int oracle_refresh_box(const int n[3], const int g[3], const int c[3], int level,
                                  const int face[3], const int child[3], int is[3], int ns[3],
                                  int id[3], int nd[3]) {
  const FaceRegion fr = make_region(n, g, c, level, face, child);
  fr.send(is, ns);
  fr.receive(id, nd);
  return 0;
}

/* fields: nblocks x 20 pointers (the slot order of the C ABI's MHD_FIELD_*;
 * NULL = absent); faces: 9 ints each (sender, receiver, level, face[3],
 * child[3]); dtype 0 = double, 1 = float. */
extern "C" int oracle_refresh_faces(int dtype, int nblocks, const int n[3], const int g[3],
                                    void* const* fields, const int* faces, int nfaces,
                                    unsigned cons) {
  return dtype == 0 ? refresh<double>(nblocks, n, g, fields, faces, nfaces, cons)
                    : refresh<float>(nblocks, n, g, fields, faces, nfaces, cons);
}
