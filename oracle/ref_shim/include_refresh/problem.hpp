/* Stand-in for Cello's problem umbrella header in the refresh checker build:
 * the Prolong / Restrict bases and their "linear" operators, with the few
 * Charm++ and Refresh names their headers mention. */
#ifndef ORACLE_SHIM_REFRESH_PROBLEM_HPP
#define ORACLE_SHIM_REFRESH_PROBLEM_HPP
#include "Cello/cello.hpp"
namespace PUP {
class able {
 public:
  able() {}
  explicit able(CkMigrateMessage*) {}
  virtual ~able() {}
  void pup(er&) {}
};
}  // namespace PUP
class Prolong;
class Refresh {
 public:
  int coarse_padding(const Prolong* prolong) const;
};
#include "problem_Prolong.hpp"
#include "problem_ProlongLinear.hpp"
#include "problem_Restrict.hpp"
#include "problem_RestrictLinear.hpp"
#define PROBLEM_HPP /* the umbrella header it stands in for reads empty */
#endif
