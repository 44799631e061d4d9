/* Minimal stand-in for the Charm++ header so that the reference's VL+CT
 * sources compile as a plain shared library (no Charm++ runtime). */
#ifndef ORACLE_SHIM_CHARM_H
#define ORACLE_SHIM_CHARM_H
#include <cstdio>
#include <string>
#include <vector>
#include <map>
#include <memory>
namespace PUP {
class er {
 public:
  bool isUnpacking() const { return false; }
  bool isPacking() const { return false; }
  bool isSizing() const { return false; }
  template <class T> er& operator|(T&) { return *this; }
};
template <class T> inline void PUParray(er&, T*, int) {}
}  // namespace PUP
class CkMigrateMessage;
#define CkPrintf printf
inline int CkMyPe() { return 0; }
inline int CkNumPes() { return 1; }
#define PUPable_decl(x)
#define PUPable_abstract(x)
#define TRACEPUP
#endif
