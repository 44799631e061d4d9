/* Stand-in for Cello's data umbrella header in the refresh checker build:
 * the Face and FaceFluxes classes only, with the buffer helpers their
 * (unused here) serialisation methods expand to.  The stand-in Block comes
 * from Cello/mesh.hpp. */
#ifndef ORACLE_SHIM_REFRESH_DATA_HPP
#define ORACLE_SHIM_REFRESH_DATA_HPP
#include <cstring>
#include <string>
#include "Cello/cello.hpp"
#ifdef CONFIG_PRECISION_SINGLE
typedef float cello_float;
#else
typedef double cello_float;
#endif
template <class T> inline void shim_save_array(char*& p, const T* a, int n) {
  std::memcpy(p, &n, sizeof(int));
  p += sizeof(int);
  std::memcpy(p, a, n * sizeof(T));
  p += n * sizeof(T);
}
template <class T> inline void shim_load_array(char*& p, T* a) {
  int n;
  std::memcpy(&n, p, sizeof(int));
  p += sizeof(int);
  std::memcpy(a, p, n * sizeof(T));
  p += n * sizeof(T);
}
#define SIZE_SCALAR_TYPE(COUNT, TYPE, VALUE) ((COUNT) += (int)sizeof(TYPE))
#define SAVE_SCALAR_TYPE(P, TYPE, VALUE) (std::memcpy((P), &(VALUE), sizeof(TYPE)), (P) += sizeof(TYPE))
#define LOAD_SCALAR_TYPE(P, TYPE, VALUE) (std::memcpy(&(VALUE), (P), sizeof(TYPE)), (P) += sizeof(TYPE))
#define SIZE_ARRAY_TYPE(COUNT, TYPE, ARRAY, SIZE) ((COUNT) += (int)(sizeof(int) + (SIZE) * sizeof(TYPE)))
#define SAVE_ARRAY_TYPE(P, TYPE, ARRAY, SIZE) shim_save_array<TYPE>((P), &(ARRAY)[0], (SIZE))
#define LOAD_ARRAY_TYPE(P, TYPE, ARRAY, SIZE) shim_load_array<TYPE>((P), &(ARRAY)[0])
#include "data_Face.hpp"
#include "data_FaceFluxes.hpp"
#define DATA_HPP /* the umbrella header it stands in for reads empty */
#endif
