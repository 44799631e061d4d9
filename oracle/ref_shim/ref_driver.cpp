/*
 * ref_driver.cpp -- TEST INFRASTRUCTURE ONLY.
 *
 * Drives the reference's own VL+CT classes (EnzoMHDIntegratorStageCommands,
 * EnzoBfieldMethodCT, the Riemann solvers, EnzoPhysicsFluidProps), compiled
 * unmodified from the Enzo-E source tree against the stand-in headers in
 * include/, so that the restated oracle can be checked against the reference
 * bit for bit.  The control flow below mirrors EnzoMethodMHDVlct::compute
 * (EnzoMethodMHDVlct.cpp:356-500) and EnzoMethodMHDVlct::timestep
 * (EnzoMethodMHDVlct.cpp:551-588) for one block held in caller arrays.
 * Built by oracle/Makefile into oracle/_ref/ only where the Enzo-E sources
 * are present; it is never shipped or called by the product.
 */
#include <cstdarg>
#include <stdexcept>

#include "Enzo/enzo.hpp"
#include "Enzo/hydro-mhd/hydro-mhd.hpp"
#include "Enzo/hydro-mhd/EnzoMHDIntegratorStageCommands.hpp"
#include "../vlct_oracle.h"

namespace {
EnzoPhysicsFluidProps* g_fluid_props = nullptr;
}

EnzoPhysicsFluidProps* enzo::fluid_props() { return g_fluid_props; }
FieldDescr* cello::field_descr() {
  static FieldDescr fd;
  return &fd;
}
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
// EnzoEOSVariant.cpp (Charm++ serialisation only) is not compiled here.
void pup(PUP::er&, EnzoEOSVariant&) noexcept {}

namespace {

struct Setup {
  EnzoPhysicsFluidProps fp;
  EnzoMHDIntegratorStageCommands* integ;
  std::string time_scheme;
  Setup(const OracleParams* p)
      : fp(p->dual_energy ? EnzoDualEnergyConfig::build_modern_formulation(p->eta)
                          : EnzoDualEnergyConfig::build_disabled(),
           EnzoFluidFloorConfig(p->density_floor, p->pressure_floor, 0.0, 0.0),
           EnzoEOSVariant(EnzoEOSIdeal::construct(p->gamma)), 0.6),
        integ(nullptr) {
    g_fluid_props = &fp;
    const char* rs[3] = {"hlle", "hllc", "hlld"};
    const char* rc[3] = {"nn", "plm", "plm_athena"};
    time_scheme = p->euler ? "euler" : "vl";
    std::vector<std::string> recon;
    if (!p->euler) recon.push_back("nn");
    recon.push_back(rc[p->recon]);
    EnzoMHDIntegratorStageArgPack args{
        rs[p->riemann], recon, p->theta_limiter,
        p->mhd ? "constrained_transport" : "no_bfield"};
    integ = new EnzoMHDIntegratorStageCommands(args);
  }
  ~Setup() {
    delete integ;
    g_fluid_props = nullptr;
  }
};

struct Views {
  std::map<std::string, CelloView<double, 3>> v;
  Views(OracleBlock* b) {
    const int mx = b->nx + 2 * b->g, my = b->ny + 2 * b->g,
              mz = b->nz + 2 * b->g;
    auto put = [&](const char* name, double* p, int ex, int ey, int ez) {
      if (p) v[name] = CelloView<double, 3>(p, mz + ez, my + ey, mx + ex);
    };
    put("density", b->rho, 0, 0, 0);
    put("velocity_x", b->vx, 0, 0, 0);
    put("velocity_y", b->vy, 0, 0, 0);
    put("velocity_z", b->vz, 0, 0, 0);
    put("total_energy", b->etot, 0, 0, 0);
    put("internal_energy", b->eint, 0, 0, 0);
    put("bfield_x", b->bx, 0, 0, 0);
    put("bfield_y", b->by, 0, 0, 0);
    put("bfield_z", b->bz, 0, 0, 0);
    put("bfieldi_x", b->bfx, 1, 0, 0);
    put("bfieldi_y", b->bfy, 0, 1, 0);
    put("bfieldi_z", b->bfz, 0, 0, 1);
    put("pressure", b->pressure, 0, 0, 0);
    put("acceleration_x", b->ax, 0, 0, 0);
    put("acceleration_y", b->ay, 0, 0, 0);
    put("acceleration_z", b->az, 0, 0, 0);
    static const char* pnames[4] = {"pass0", "pass1", "pass2", "pass3"};
    for (int k = 0; k < b->npassive && k < 4; k++) put(pnames[k], b->passive[k], 0, 0, 0);
  }
  EnzoEFltArrayMap map(const str_vec_t& keys) {
    std::vector<EFlt3DArray> arrs;
    for (const auto& k : keys) arrs.push_back(v.at(k));
    return EnzoEFltArrayMap("integration", keys, arrs);
  }
};

// Same construction as EnzoVlctScratchSpace (EnzoMethodMHDVlct.hpp:217-312).
struct Scratch {
  CelloView<enzo_float, 3> interface_vel_arr;
  EnzoEFltArrayMap temp_integration_map, primitive_map, priml_map, primr_map,
      xflux_map, yflux_map, zflux_map, dUcons_map;
  Scratch(const std::array<int, 3>& shape, const str_vec_t& integ_keys,
          const str_vec_t& prim_keys, const str_vec_t& du_keys, bool de)
      : interface_vel_arr(de ? EFlt3DArray(shape[0], shape[1], shape[2])
                             : EFlt3DArray()) {
    auto setup = [&shape](const std::string& name,
                          const std::array<int, 3>& centering,
                          const str_vec_t& keys) {
      std::array<int, 3> cur(shape);
      for (int i = 0; i < 3; i++) cur[i] += centering[i];
      return EnzoEFltArrayMap(name, keys, cur);
    };
    temp_integration_map = setup("temp_integration", {0, 0, 0}, integ_keys);
    xflux_map = setup("xflux", {0, 0, -1}, integ_keys);
    yflux_map = setup("yflux", {0, -1, 0}, integ_keys);
    zflux_map = setup("zflux", {-1, 0, 0}, integ_keys);
    dUcons_map = setup("dUcons", {0, 0, 0}, du_keys);
    primitive_map = setup("primitive", {0, 0, 0}, prim_keys);
    priml_map = setup("priml", {0, 0, 0}, prim_keys);
    primr_map = setup("primr", {0, 0, 0}, prim_keys);
  }
};

}  // namespace

// The reference's own save_fluxes_for_corrections_ loop
// (EnzoMethodMHDVlct.cpp:250-330), reading its flux maps after the final
// stage; out and quantities as in oracle_step_fc.
static void save_fc(const std::array<EnzoEFltArrayMap, 3>& flux_maps, int g,
                    const int cc[3], const double cw[3], double dt,
                    double* const* out, int nq, const int* quantities) {
  static const char* names[10] = {"density", "velocity_x", "velocity_y",
                                  "velocity_z", "total_energy", "internal_energy",
                                  "pass0", "pass1", "pass2", "pass3"};
  const int n[3] = {cc[0] - 2 * g, cc[1] - 2 * g, cc[2] - 2 * g};
  for (int dim = 0; dim < 3; dim++) {
    const double dt_dxi = dt / cw[dim];
    for (int iq = 0; iq < nq; iq++) {
      CelloView<const enzo_float, 3> flux_arr = flux_maps[dim].at(names[quantities[iq]]);
      double* left = out[(dim * 2 + 0) * nq + iq];
      double* right = out[(dim * 2 + 1) * nq + iq];
      if (dim == 0) {
        const int left_ix = g - 1, right_ix = cc[0] - g - 1;
        for (int iz = 0; iz < n[2]; iz++)
          for (int iy = 0; iy < n[1]; iy++) {
            if (left) left[iz * n[1] + iy] = dt_dxi * flux_arr(g + iz, g + iy, left_ix);
            if (right) right[iz * n[1] + iy] = dt_dxi * flux_arr(g + iz, g + iy, right_ix);
          }
      } else if (dim == 1) {
        const int left_iy = g - 1, right_iy = cc[1] - g - 1;
        for (int iz = 0; iz < n[2]; iz++)
          for (int ix = 0; ix < n[0]; ix++) {
            if (left) left[iz * n[0] + ix] = dt_dxi * flux_arr(g + iz, left_iy, g + ix);
            if (right) right[iz * n[0] + ix] = dt_dxi * flux_arr(g + iz, right_iy, g + ix);
          }
      } else {
        const int left_iz = g - 1, right_iz = cc[2] - g - 1;
        for (int iy = 0; iy < n[1]; iy++)
          for (int ix = 0; ix < n[0]; ix++) {
            if (left) left[iy * n[0] + ix] = dt_dxi * flux_arr(left_iz, g + iy, g + ix);
            if (right) right[iy * n[0] + ix] = dt_dxi * flux_arr(right_iz, g + iy, g + ix);
          }
      }
    }
  }
}

static int ref_step_impl(const OracleParams* p, OracleBlock* b, double dt,
                         double* const* fc_out, int fc_nq, const int* fc_q);

extern "C" int ref_step(const OracleParams* p, OracleBlock* b, double dt) {
  return ref_step_impl(p, b, dt, nullptr, 0, nullptr);
}

extern "C" int ref_step_fc(const OracleParams* p, OracleBlock* b, double dt,
                           double* const* out, int nq, const int* quantities) {
  return ref_step_impl(p, b, dt, out, nq, quantities);
}

static int ref_step_impl(const OracleParams* p, OracleBlock* b, double dt,
                         double* const* fc_out, int fc_nq, const int* fc_q) {
  try {
    Setup s(p);
    Views views(b);
    EnzoBlock block;
    block.data_.field_.views = &views.v;
    block.CellWidth[0] = b->dx;
    block.CellWidth[1] = b->dy;
    block.CellWidth[2] = b->dz;

    // passive scalars (the lazy passive list of EnzoMethodMHDVlct::compute,
    // :366) travel in every map after the integration quantities
    str_vec_t passive_list;
    for (int k = 0; k < b->npassive && k < 4; k++)
      passive_list.push_back("pass" + std::to_string(k));
    auto with_passive = [&](str_vec_t keys) {
      keys.insert(keys.end(), passive_list.begin(), passive_list.end());
      return keys;
    };
    const str_vec_t integ_keys = with_passive(s.integ->integration_quantity_keys());
    const str_vec_t prim_keys = with_passive(s.integ->primitive_quantity_keys());
    EnzoEFltArrayMap external = views.map(integ_keys);
    const std::array<int, 3> shape = {external.array_shape(0),
                                      external.array_shape(1),
                                      external.array_shape(2)};
    const bool de = p->dual_energy != 0;
    Scratch scratch(shape, integ_keys, prim_keys,
                    with_passive(s.integ->dUcons_map_keys()), de);
    std::array<EnzoEFltArrayMap, 3> flux_maps = {
        scratch.xflux_map, scratch.yflux_map, scratch.zflux_map};
    // get_accel_map_ (EnzoMethodMHDVlct.cpp:219-233): empty without the
    // acceleration fields
    const EnzoEFltArrayMap accel_map =
        (b->ax && b->ay && b->az)
            ? views.map({"acceleration_x", "acceleration_y", "acceleration_z"})
            : EnzoEFltArrayMap();
    EFlt3DArray interface_vel_arr = scratch.interface_vel_arr;
    const int nstages = p->euler ? 1 : 2;
    EnzoBfieldMethod* bfield = s.integ->construct_bfield_method(nstages);
    if (bfield) bfield->register_target_block(&block);
    const std::array<enzo_float, 3> cw = {block.CellWidth[0],
                                          block.CellWidth[1],
                                          block.CellWidth[2]};
    int stale_depth = 0;
    for (int stage = 0; stage < nstages; stage++) {
      const bool is_final = (stage + 1) == nstages;
      const double cur_dt = (!is_final) ? dt / 2. : dt;
      EnzoEFltArrayMap cur = (stage == 0) ? external
                                          : scratch.temp_integration_map;
      EnzoEFltArrayMap out = is_final ? external : scratch.temp_integration_map;
      s.integ->compute_update_stage(
          external, cur, out, scratch.primitive_map, scratch.priml_map,
          scratch.primr_map, flux_maps, scratch.dUcons_map, accel_map,
          interface_vel_arr, passive_list, bfield, (unsigned short)stage,
          cur_dt, stale_depth, cw);
      stale_depth += s.integ->staling_from_stage(stage);
      if (bfield) bfield->increment_partial_timestep();
      if (is_final && fc_out) {
        const int cc[3] = {shape[2], shape[1], shape[0]};
        const double cwd[3] = {b->dx, b->dy, b->dz};
        save_fc(flux_maps, b->g, cc, cwd, dt, fc_out, fc_nq, fc_q);
      }
    }
    delete bfield;
  } catch (const std::exception& e) {
    fprintf(stderr, "ref_step: %s\n", e.what());
    return 1;
  }
  return 0;
}

extern "C" double ref_timestep(const OracleParams* p, OracleBlock* b) {
  try {
    Setup s(p);
    Views views(b);
    EnzoEFltArrayMap integ = views.map(s.integ->integration_quantity_keys());
    if (s.fp.dual_energy_config().any_enabled()) {
      s.fp.apply_floor_to_energy_and_sync(integ, 0);
    }
    CelloView<enzo_float, 3> pressure = views.v.at("pressure");
    s.fp.pressure_from_integration(integ, pressure, 0);
    double dt = s.integ->timestep(integ, pressure, b->dx, b->dy, b->dz);
    return dt * p->courant;
  } catch (const std::exception& e) {
    fprintf(stderr, "ref_timestep: %s\n", e.what());
    return -1.0;
  }
}

// Cell-centred B from face B over a whole block, through the reference's
// EnzoBfieldMethodCT::compute_center_bfield (EnzoBfieldMethodCT.cpp:702-728)
// with stale depth 0, as EnzoInitialBCenter::initialize_bfield_center does.
extern "C" int ref_center_bfield(int mx, int my, int mz, double* bfx, double* bfy,
                                 double* bfz, double* bx, double* by, double* bz) {
  try {
    double* bi[3] = {bfx, bfy, bfz};
    double* bc[3] = {bx, by, bz};
    for (int dim = 0; dim < 3; dim++) {
      CelloView<enzo_float, 3> c(bc[dim], mz, my, mx);
      CelloView<enzo_float, 3> f(bi[dim], mz + (dim == 2), my + (dim == 1), mx + (dim == 0));
      CelloView<const enzo_float, 3> fc = f;
      EnzoBfieldMethodCT::compute_center_bfield(dim, c, fc, 0);
    }
  } catch (const std::exception& e) {
    fprintf(stderr, "ref_center_bfield: %s\n", e.what());
    return 1;
  }
  return 0;
}
