/* Stand-in for hydro-mhd.hpp: the VL+CT toolkit and Riemann solvers only
 * (the Method classes of the full header need the Cello runtime). */
#ifndef ORACLE_SHIM_HYDROMHD_HPP
#define ORACLE_SHIM_HYDROMHD_HPP
#include "Enzo/enzo.hpp"
#include "Enzo/hydro-mhd/toolkit/toolkit.hpp"
#include "Enzo/hydro-mhd/riemann/EnzoRiemann.hpp"
#endif
