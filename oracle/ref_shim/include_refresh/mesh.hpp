/* Stand-in for Cello's mesh umbrella header in the refresh checker build:
 * only the Box class (mesh_Box.hpp) on top of the oracle's shim. */
#ifndef ORACLE_SHIM_REFRESH_MESH_HPP
#define ORACLE_SHIM_REFRESH_MESH_HPP
#include "Cello/cello.hpp"
#include "mesh_Box.hpp"
#define MESH_HPP /* the umbrella header it stands in for reads empty */
#endif
