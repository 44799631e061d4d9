/* Minimal stand-in for Cello's umbrella header (oracle build only). */
#ifndef ORACLE_SHIM_CELLO_HPP
#define ORACLE_SHIM_CELLO_HPP
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <functional>
#include <limits>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>
#include "charm++.h"
#include "_error.hpp"
#include "cello_defines.hpp"
#include "_view.hpp"
namespace cello {
inline int rank() { return 3; }
const double pi = 3.14159265358979324;
}
#ifndef MIN
#define MIN(A, B) ((A) < (B) ? (A) : (B))
#endif
#ifndef MAX
#define MAX(A, B) ((A) > (B) ? (A) : (B))
#endif
#include "Cello/mesh.hpp"
#endif
