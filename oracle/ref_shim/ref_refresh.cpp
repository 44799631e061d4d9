/*
 * ref_refresh.cpp -- TEST INFRASTRUCTURE ONLY.
 *
 * Drives the reference's own refresh pieces -- Box (src/Cello/mesh_Box.cpp),
 * ProlongLinear and RestrictLinear (src/Cello/problem_ProlongLinear.cpp,
 * problem_RestrictLinear.cpp), compiled unmodified -- through the control
 * flow of FieldFace::face_to_face (src/Cello/data_FieldFace.cpp:440-566) with
 * the Box set up as FieldFace::set_box_ and box_adjust_accumulate_ do
 * (data_FieldFace.cpp:982-1018) for a face created by
 * Block::refresh_load_field_face_ (control_refresh.cpp:331-360: no ghost
 * flags, not accumulating).  Density weighting multiplies and divides the
 * sender's cells in place exactly as mul_by_density_ / div_by_density_ do
 * (data_FieldFace.cpp:863-980).  It also exposes FaceFluxes::coarsen
 * (data_FaceFluxes.cpp:128-252), the flux coarsening of the flux
 * correction.  Built into oracle/_ref/ only where the
 * Enzo-E sources are present; never shipped or called by the product.
 */
#include <cstdarg>
#include <stdexcept>

#include "include_refresh/mesh.hpp"
#include "include_refresh/problem.hpp"
#include "include_refresh/data.hpp"

void cello::message(FILE* fp, const char* type, const char* file, int line,
                    const char* function, const char* message, ...) {
  va_list args;
  va_start(args, message);
  fprintf(fp, "%s %s:%d %s: ", type, file, line, function);
  vfprintf(fp, message, args);
  fprintf(fp, "\n");
  va_end(args);
}
void cello::error() { throw std::runtime_error("cello::error"); }
int Refresh::coarse_padding(const Prolong* prolong) const {
  return prolong->coarse_padding_();
}

namespace {

enum { SAME = 0, FINE = 1, COARSE = -1 };

// FieldFace::set_box_ then box_adjust_accumulate_ (accumulate false, ghost_
// flags 0), then the two get_start_size calls of face_to_face
void boxes(int n3[3], int g3[3], int c3[3], int type, int face[3], int child[3],
           Prolong* prolong, int is3[3], int ns3[3], int id3[3], int nd3[3]) {
  Box box(3, n3, g3);
  box.set_block(BoxType_receive, type, face, child);
  Refresh refresh;
  int pad = prolong ? refresh.coarse_padding(prolong) : 0;
  if (type != FINE) pad = 0;
  box.set_padding(pad);
  box.compute_region();
  box.set_centering(c3);
  int gs3[3] = {0, 0, 0};
  box.set_send_ghosts(gs3);
  box.compute_block_start(BoxType_receive);
  box.compute_region();
  box.get_start_size(is3, ns3, BlockType::send, BlockType::send, true);
  box.get_start_size(id3, nd3, BlockType::receive, BlockType::receive, false);
}

template <class T>
void scale(T* f, const T* d, const int i3[3], const int n3[3], const int m3[3], bool mul) {
  for (int iz = i3[2]; iz < i3[2] + n3[2]; iz++)
    for (int iy = i3[1]; iy < i3[1] + n3[1]; iy++)
      for (int ix = i3[0]; ix < i3[0] + n3[0]; ix++) {
        const int i = ix + m3[0] * (iy + m3[1] * iz);
        if (mul)
          f[i] *= d[i];
        else
          f[i] /= d[i];
      }
}

template <class T>
int refresh_faces(int nblocks, const int n[3], const int g[3], void* const* fields,
                  const int* faces, int nfaces, unsigned cons) {
  const int NSLOT = 20, NCELL = 17;
  ProlongLinear prolong;
  RestrictLinear restrict_op;
  const precision_type prec = sizeof(T) == 8 ? precision_double : precision_single;
  for (int k = 0; k < nfaces; k++) {
    const int* fc = faces + 9 * k;
    const int s = fc[0], r = fc[1], type = fc[2];
    int face[3] = {fc[3], fc[4], fc[5]}, child[3] = {fc[6], fc[7], fc[8]};
    if (s < 0 || s >= nblocks || r < 0 || r >= nblocks) return 1;
    void* const* sf = fields + (size_t)NSLOT * s;
    void* const* rf = fields + (size_t)NSLOT * r;
    // field list order: the cell fields (density first), then bfieldi
    for (int slot = 0; slot < NSLOT; slot++) {
      if (!sf[slot]) continue;
      int c3[3] = {0, 0, 0};
      if (slot >= NCELL) {
        if (type != SAME) return 2;
        c3[slot - NCELL] = 1;
      }
      int n3[3] = {n[0], n[1], n[2]}, g3[3] = {g[0], g[1], g[2]};
      int m3[3] = {n[0] + 2 * g[0] + c3[0], n[1] + 2 * g[1] + c3[1], n[2] + 2 * g[2] + c3[2]};
      int is3[3], ns3[3], id3[3], nd3[3];
      boxes(n3, g3, c3, type, face, child, &prolong, is3, ns3, id3, nd3);
      T* src = (T*)sf[slot];
      T* dst = (T*)rf[slot];
      const bool weighted = type != SAME && ((cons >> slot) & 1u);
      if (weighted) scale<T>(src, (const T*)sf[0], is3, ns3, m3, true);
      if (type == FINE) {
        bool need_padding = (g3[0] % 2 == 1) || (g3[1] % 2 == 1) || (g3[2] % 2 == 1);
        if (need_padding) return 3;
        prolong.apply(prec, dst, m3, id3, nd3, src, m3, is3, ns3, false);
      } else if (type == COARSE) {
        restrict_op.apply(prec, dst, m3, id3, nd3, src, m3, is3, ns3, false);
      } else {
        // FieldFace::copy_ (data_FieldFace.cpp:806-841), not accumulating
        const int is0 = is3[0] + m3[0] * (is3[1] + m3[1] * is3[2]);
        const int id0 = id3[0] + m3[0] * (id3[1] + m3[1] * id3[2]);
        for (int iz = 0; iz < ns3[2]; iz++)
          for (int iy = 0; iy < ns3[1]; iy++)
            for (int ix = 0; ix < ns3[0]; ix++) {
              const int o = ix + m3[0] * (iy + m3[1] * iz);
              dst[id0 + o] = src[is0 + o];
            }
      }
      if (weighted) {
        scale<T>(src, (const T*)sf[0], is3, ns3, m3, false);
        scale<T>(dst, (const T*)rf[0], id3, nd3, m3, false);
      }
    }
  }
  return 0;
}

}  // namespace

extern "C" int ref_refresh_box(const int n[3], const int g[3], const int c[3], int type,
                               const int face[3], const int child[3], int is3[3],
                               int ns3[3], int id3[3], int nd3[3]) {
  try {
    int n3[3] = {n[0], n[1], n[2]}, g3[3] = {g[0], g[1], g[2]}, c3[3] = {c[0], c[1], c[2]};
    int f3[3] = {face[0], face[1], face[2]}, ch3[3] = {child[0], child[1], child[2]};
    ProlongLinear prolong;
    boxes(n3, g3, c3, type, f3, ch3, &prolong, is3, ns3, id3, nd3);
  } catch (const std::exception& e) {
    fprintf(stderr, "ref_refresh_box: %s\n", e.what());
    return -1;
  }
  return 0;
}

extern "C" int ref_refresh_faces(int dtype, int nblocks, const int n[3], const int g[3],
                                 void* const* fields, const int* faces, int nfaces,
                                 unsigned cons) {
  try {
    return dtype == 0 ? refresh_faces<double>(nblocks, n, g, fields, faces, nfaces, cons)
                      : refresh_faces<float>(nblocks, n, g, fields, faces, nfaces, cons);
  } catch (const std::exception& e) {
    fprintf(stderr, "ref_refresh_faces: %s\n", e.what());
    return -1;
  }
}

// FaceFluxes::coarsen of one fine face array: a FaceFluxes on the given axis
// face of a block of n cells, filled with `fine` (inner index fastest), then
// coarsened for the child index c3; out receives the array after the call.
extern "C" int ref_coarsen_fluxes(const int n[3], int axis, int face, const int c3[3],
                                  const double* fine, double* out) {
  try {
    int f3[3] = {0, 0, 0};
    f3[axis] = face == 0 ? -1 : 1;
    Face fc(f3[0], f3[1], f3[2], axis, face);
    FaceFluxes ff(fc, 0, n[0], n[1], n[2], 0, 0, 0);
    ff.allocate_storage();
    int mx, my, mz;
    const int m = ff.get_size(&mx, &my, &mz);
    double* a = ff.flux_array();
    for (int i = 0; i < m; i++) a[i] = fine[i];
    ff.coarsen(c3[0], c3[1], c3[2], 3);
    for (int i = 0; i < m; i++) out[i] = a[i];
  } catch (const std::exception& e) {
    fprintf(stderr, "ref_coarsen_fluxes: %s\n", e.what());
    return -1;
  }
  return 0;
}
