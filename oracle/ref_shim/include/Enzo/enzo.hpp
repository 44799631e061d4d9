/* Minimal stand-in for Enzo's umbrella header: the typedefs, the global
 * accessors (enzo::fluid_props(), enzo::block()) and the headers that the
 * VL+CT toolkit, Riemann solvers and fluid-props sources use. */
#ifndef ORACLE_SHIM_ENZO_HPP
#define ORACLE_SHIM_ENZO_HPP
#include "Cello/cello.hpp"
#include "Enzo/enzo_typedefs.hpp"
class EnzoPhysicsFluidProps;
class EnzoMethodGrackle;
class EnzoPhysicsCosmology;
class EnzoBlock : public Block {
 public:
  enzo_float CellWidth[3];
};
namespace enzo {
EnzoPhysicsFluidProps* fluid_props();
inline const EnzoMethodGrackle* grackle_method() { return nullptr; }
inline EnzoBlock* block(Block* b) { return static_cast<EnzoBlock*>(b); }
}
#include "Enzo/utils/utils.hpp"
#include "Enzo/utils/EnzoPermutedCoordinates.hpp"
#include "Enzo/fluid-props/fluid-props.hpp"
class EnzoMethodGrackle {
 public:
  void calculate_pressure(const EnzoFieldAdaptor&, enzo_float*, int) const {}
};
#endif
