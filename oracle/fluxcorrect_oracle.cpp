/*
 * fluxcorrect_oracle.cpp -- TEST INFRASTRUCTURE ONLY.
 *
 * A CPU restatement of Cello's flux correction at coarse-fine faces, in the
 * reference's loop structure and operation order (compiled with
 * -ffp-contract=off):
 *  - FaceFluxes::coarsen (src/Cello/data_FaceFluxes.cpp:128-252, rank 3):
 *    a zeroed copy of the fine face array receives, for every fine face in
 *    (outer, inner) order, four adds of 0.25 * dArea * flux (dArea = 0.125)
 *    at the coarse face covering it, offset by the child's quadrant;
 *  - FluxData::sum_neighbor_fluxes (data_FluxData.hpp:136-145): the
 *    coarsened arrays of the four children summed into a zeroed array;
 *  - MethodFluxCorrect::flux_correct_ and flux_correct_helper_ /
 *    divide_flux_corrected_cells_by_density_
 *    (src/Cello/problem_MethodFluxCorrect.cpp:293-558).
 * No code here is shared with the CUDA product.
 */
#include <cstddef>
#include <vector>

namespace {

// density, velocity_x/y/z, total_energy, internal_energy, passive scalars 0-3
// (every field of the reference's flux-correction group,
// src/Cello/problem_MethodFluxCorrect.cpp:55-77)
const int NQ = 10;

template <class T>
T* fluxp(void* const* fluxes, int blk, int axis, int side, int q) {
  return (T*)fluxes[((size_t)blk * 3 + axis) * 2 * NQ + side * NQ + q];
}

// the face array's transverse axes: inner (fastest) and outer
void transverse(int axis, int& a_in, int& a_out) {
  a_in = axis == 0 ? 1 : 0;
  a_out = axis == 2 ? 1 : 2;
}

// FaceFluxes::coarsen of one fine face array (ni x no, inner fastest) of a
// child with transverse child index (ci, co); out receives the full-size
// coarsened array (zero outside the child's quarter).
template <class T>
void coarsen(const T* fine, int ni, int no, int ci, int co, T* out) {
  for (int i = 0; i < ni * no; i++) out[i] = 0.0;
  const int hi = ni / 2, ho = no / 2;  // the reference's m?c = n?_/2 + c?_ with c?_ = 0
  const int i0 = ci * hi, o0 = co * ho * ni;
  const T darea = 0.125;
  for (int of = 0; of < no; of++) {
    const int ocm = ni * (of >> 1), ocp = ni * ((of + 0) >> 1);
    for (int inf = 0; inf < ni; inf++) {
      const int icm = inf >> 1, icp = (inf + 0) >> 1;
      const T f = fine[inf + ni * of];
      out[i0 + o0 + ocm + icm] += 0.25 * darea * f;
      out[i0 + o0 + ocm + icp] += 0.25 * darea * f;
      out[i0 + o0 + ocp + icm] += 0.25 * darea * f;
      out[i0 + o0 + ocp + icp] += 0.25 * darea * f;
    }
  }
}

template <class T>
int flux_correct(int nblocks, const int n[3], const int g[3], void* const* fields,
                 void* const* fluxes, const int* faces, int nfaces, unsigned cons) {
  const int m[3] = {n[0] + 2 * g[0], n[1] + 2 * g[1], n[2] + 2 * g[2]};
  // children of every (coarse block, axis, face): [outer][inner]
  std::vector<int> child((size_t)nblocks * 6 * 4, -1);
  std::vector<char> finer((size_t)nblocks * 6, 0);
  for (int k = 0; k < nfaces; k++) {
    const int* f = faces + 9 * k;
    const int s = f[0], r = f[1], type = f[2];
    const int nz = (f[3] != 0) + (f[4] != 0) + (f[5] != 0);
    if (type != -1 || nz != 1) continue;
    const int axis = f[3] ? 0 : (f[4] ? 1 : 2);
    const int face = f[3 + axis] == 1 ? 0 : 1;
    int a_in, a_out;
    transverse(axis, a_in, a_out);
    const int ci = f[6 + a_in], co = f[6 + a_out];
    child[(((size_t)r * 6 + axis * 2 + face) * 2 + co) * 2 + ci] = s;
    finer[(size_t)r * 6 + axis * 2 + face] = 1;
  }
  std::vector<T> coarse, nbr, old_rho, temp;
  for (int b = 0; b < nblocks; b++) {
    bool any = false;
    for (int k = 0; k < 6; k++) any = any || finer[(size_t)b * 6 + k];
    if (!any) continue;
    // the quantities stored (the same on every face)
    bool stored[NQ];
    for (int q = 0; q < NQ; q++) stored[q] = fluxp<T>(fluxes, b, 0, 0, q) != nullptr;
    // neighbour fluxes: FluxData::sum_neighbor_fluxes of the four children
    std::vector<std::vector<T>> neighbour(6 * NQ);
    for (int k = 0; k < 6; k++) {
      if (!finer[(size_t)b * 6 + k]) continue;
      const int axis = k >> 1, face = k & 1;
      int a_in, a_out;
      transverse(axis, a_in, a_out);
      const int ni = n[a_in], no = n[a_out];
      for (int q = 0; q < NQ; q++) {
        if (!stored[q]) continue;
        nbr.assign((size_t)ni * no, T(0));
        coarse.resize((size_t)ni * no);
        for (int co = 0; co < 2; co++)
          for (int ci = 0; ci < 2; ci++) {
            const int c = child[(((size_t)b * 6 + k) * 2 + co) * 2 + ci];
            if (c < 0) return 1;
            coarsen<T>(fluxp<T>(fluxes, c, axis, 1 - face, q), ni, no, ci, co, coarse.data());
            for (int i = 0; i < ni * no; i++) nbr[i] += coarse[i];
          }
        neighbour[k * NQ + q] = nbr;
      }
    }
    // MethodFluxCorrect::flux_correct_: indices relative to the first active
    // cell, as field.unknowns() gives them
    T* const* f = (T* const*)(fields + (size_t)b * NQ);
    const size_t act = (size_t)g[0] + (size_t)m[0] * (g[1] + (size_t)m[1] * g[2]);
    auto helper = [&](T* arr, int q) {  // flux_correct_helper_
      for (int axis = 0; axis < 3; axis++)
        for (int face = 0; face < 2; face++) {
          if (!finer[(size_t)b * 6 + axis * 2 + face]) continue;
          int a_in, a_out;
          transverse(axis, a_in, a_out);
          const T* fb = fluxp<T>(fluxes, b, axis, face, q);
          const T* fn = neighbour[(axis * 2 + face) * NQ + q].data();
          const int ni = n[a_in];
          int c[3];
          c[axis] = face == 0 ? 0 : n[axis] - 1;
          for (c[a_out] = 0; c[a_out] < n[a_out]; c[a_out]++)
            for (c[a_in] = 0; c[a_in] < n[a_in]; c[a_in]++) {
              const size_t i = c[0] + (size_t)m[0] * (c[1] + (size_t)m[1] * c[2]);
              const size_t j = c[a_in] + (size_t)ni * c[a_out];
              arr[i] += (2 * face - 1) * (fb[j] - fn[j]);
            }
        }
    };
    const size_t nm = (size_t)m[0] * m[1] * m[2];
    old_rho.assign(nm, T(0));
    temp.assign(nm, T(0));
    T* rho = f[0] + act;
    T* orho = old_rho.data() + act;
    for (int z = 0; z < n[2]; z++)
      for (int y = 0; y < n[1]; y++)
        for (int x = 0; x < n[0]; x++) {
          const size_t i = x + (size_t)m[0] * (y + (size_t)m[1] * z);
          orho[i] = rho[i];
        }
    if (stored[0]) helper(rho, 0);
    for (int q = 1; q < NQ; q++) {
      if (!stored[q]) continue;
      T* u = f[q] + act;
      if ((cons >> q) & 1u) {
        T* t = temp.data() + act;
        for (int z = 0; z < n[2]; z++)
          for (int y = 0; y < n[1]; y++)
            for (int x = 0; x < n[0]; x++) {
              const size_t i = x + (size_t)m[0] * (y + (size_t)m[1] * z);
              t[i] = orho[i] * u[i];
            }
        helper(t, q);
        // divide_flux_corrected_cells_by_density_
        for (int axis = 0; axis < 3; axis++)
          for (int face = 0; face < 2; face++) {
            if (!finer[(size_t)b * 6 + axis * 2 + face]) continue;
            int a_in, a_out;
            transverse(axis, a_in, a_out);
            int c[3];
            c[axis] = face == 0 ? 0 : n[axis] - 1;
            for (c[a_out] = 0; c[a_out] < n[a_out]; c[a_out]++)
              for (c[a_in] = 0; c[a_in] < n[a_in]; c[a_in]++) {
                const size_t i = c[0] + (size_t)m[0] * (c[1] + (size_t)m[1] * c[2]);
                u[i] = t[i] / rho[i];
              }
          }
      } else {
        helper(u, q);
      }
    }
  }
  return 0;
}

}  // namespace

/* fields: nblocks x 10 pointers (density, velocity_x/y/z, total_energy,
 * internal_energy, passive scalars 0-3; NULL = absent); cons: bits of the
 * same slots; fluxes: nblocks x 3 x 2 x 10 pointers of the
 * stored boundary fluxes (axis, side, quantity); faces: 9 ints each (the mesh
 * refresh faces); dtype 0 = double, 1 = float. */
extern "C" int oracle_flux_correct(int dtype, int nblocks, const int n[3], const int g[3],
                                   void* const* fields, void* const* fluxes, const int* faces,
                                   int nfaces, unsigned cons) {
  return dtype == 0
             ? flux_correct<double>(nblocks, n, g, fields, fluxes, faces, nfaces, cons)
             : flux_correct<float>(nblocks, n, g, fields, fluxes, faces, nfaces, cons);
}

extern "C" void oracle_coarsen_fluxes(int dtype, int ni, int no, const void* fine, int ci,
                                      int co, void* out) {
  if (dtype == 0)
    coarsen<double>((const double*)fine, ni, no, ci, co, (double*)out);
  else
    coarsen<float>((const float*)fine, ni, no, ci, co, (float*)out);
}
