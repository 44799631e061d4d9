/* stand-in: no Grackle in the oracle build */
#ifndef ORACLE_SHIM_CHEMISTRY_HPP
#define ORACLE_SHIM_CHEMISTRY_HPP
struct grackle_field_data;
#endif
