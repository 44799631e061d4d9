// mhdvlct_method.hpp -- C++ host side of the GB300 VL+CT step, mirroring the
// reference's Method plugin (src/Cello/problem_Method.hpp:23-124 and
// src/Enzo/hydro-mhd/EnzoMethodMHDVlct.hpp).
//
// EnzoMethodMHDVlctGB300 keeps the reference's surface: it is constructed
// from the `Method:mhd_vlct` parameter block (plus Physics:fluid_props),
// name() is "mhd_vlct", compute(block) advances one block by the block's dt,
// timestep(block) returns courant * CFL dt of the whole ghosted block.  A
// block is described by `MhdBlockView` (device pointers in Cello's field
// layout).  Where the reference calls ERROR (fatal), this class throws
// mhdvlct::Error carrying the C ABI status and message.
//
// Header-only over include/mhdvlct_gb300.h; link with -lmhdvlct_gb300.
#ifndef MHDVLCT_METHOD_HPP
#define MHDVLCT_METHOD_HPP

#include <stdexcept>
#include <string>
#include <vector>

#include "mhdvlct_gb300.h"

namespace mhdvlct {

class Error : public std::runtime_error {
 public:
  Error(int code, const std::string& msg)
      : std::runtime_error("[" + std::to_string(code) + "] " + msg), code_(code) {}
  int code() const noexcept { return code_; }

 private:
  int code_;
};

// A block handed to the Method: the field pointers (device memory, Cello
// layout) plus the block's dt, as Cello's Block carries them
// (Block::dt(), src/Cello/mesh_Block.hpp:115).
struct Block {
  MhdBlockView fields;
  double dt = 0.0;
  bool is_leaf = true;
};

class EnzoMethodMHDVlctGB300 {
 public:
  // From a parameter text in Cello's syntax (Method:mhd_vlct, Physics:...).
  explicit EnzoMethodMHDVlctGB300(const std::string& parameter_text) {
    MhdVlctParams p;
    char err[256] = {0};
    const int rc = mhdvlct_params_parse(parameter_text.c_str(), &p, err, sizeof(err));
    if (rc != MHD_OK) throw Error(rc, err);
    create_(p);
  }
  explicit EnzoMethodMHDVlctGB300(const MhdVlctParams& p) { create_(p); }
  ~EnzoMethodMHDVlctGB300() {
    if (h_) mhdvlct_destroy(h_);
  }
  EnzoMethodMHDVlctGB300(const EnzoMethodMHDVlctGB300&) = delete;
  EnzoMethodMHDVlctGB300& operator=(const EnzoMethodMHDVlctGB300&) = delete;

  // Method::name (EnzoMethodMHDVlct.hpp)
  std::string name() const { return "mhd_vlct"; }
  // Method::courant
  double courant() const { return mhdvlct_courant(h_); }
  int required_ghost_depth() const { return mhdvlct_required_ghost_depth(h_); }

  // Method::compute (EnzoMethodMHDVlct.cpp:356-500).  Non-leaf blocks are
  // skipped as in the reference (:364); the caller then continues as
  // Block::compute_done() would.
  void compute(Block& b, void* stream = nullptr) {
    if (!b.is_leaf) return;
    check_(mhdvlct_block_step(h_, &b.fields, b.dt, stream));
  }

  // Method::timestep (EnzoMethodMHDVlct.cpp:551-588).
  double timestep(Block& b, void* stream = nullptr) {
    double dt = 0.0;
    check_(mhdvlct_block_timestep(h_, &b.fields, &dt, stream));
    return dt;
  }

  // The ghost refresh Cello performs before compute, for a single periodic
  // block (neighbour == itself).
  void refresh_periodic(Block& b, void* stream = nullptr) {
    check_(mhdvlct_fill_ghosts_periodic(h_, &b.fields, stream));
  }

  // Method::compute with store_fluxes_for_corrections
  // (EnzoMethodMHDVlct.cpp:136-141, 250-330): the step also writes the
  // dt/dx-scaled boundary fluxes into `fc` (Cello's FluxData, on the device).
  void compute_store_fluxes(Block& b, const MhdFluxCorrection& fc, void* stream = nullptr) {
    if (!b.is_leaf) return;
    check_(mhdvlct_block_step_fc(h_, &b.fields, b.dt, &fc, stream));
  }

  // The ghost refresh of a mesh's leaves whose neighbours may be one level
  // coarser or finer (Block::refresh_load_field_faces_ with the "linear"
  // prolongation and restriction), all faces in one launch.
  void refresh(const std::vector<Block>& blocks, const std::vector<MhdRefreshFace>& faces,
               unsigned conservative = MHD_CONSERVATIVE_DEFAULT, void* stream = nullptr) {
    const std::vector<MhdBlockView> v = views_(blocks);
    check_(mhdvlct_refresh_faces(h_, v.data(), (int)v.size(), faces.data(), (int)faces.size(),
                                 conservative, stream));
  }

  // Cello's "flux_correct" Method over the leaves after compute_store_fluxes
  // (MethodFluxCorrect::compute, src/Cello/problem_MethodFluxCorrect.cpp).
  void flux_correct(const std::vector<Block>& blocks,
                    const std::vector<MhdFluxCorrection>& fluxes,
                    const std::vector<MhdRefreshFace>& faces,
                    unsigned conservative = MHD_CONSERVATIVE_DEFAULT, void* stream = nullptr) {
    if (fluxes.size() != blocks.size()) throw Error(MHD_ERR_INVALID, "one flux set per block");
    const std::vector<MhdBlockView> v = views_(blocks);
    check_(mhdvlct_flux_correct(h_, v.data(), (int)v.size(), fluxes.data(), faces.data(),
                                (int)faces.size(), conservative, stream));
  }

  mhdvlct_handle* handle() const noexcept { return h_; }

 private:
  void create_(const MhdVlctParams& p) {
    mhdvlct_handle* h = nullptr;
    const int rc = mhdvlct_create(&p, &h);
    if (rc != MHD_OK) {
      const std::string m = h ? mhdvlct_last_error_string(h) : "mhdvlct_create";
      if (h) mhdvlct_destroy(h);
      throw Error(rc, m);
    }
    h_ = h;
  }
  static std::vector<MhdBlockView> views_(const std::vector<Block>& blocks) {
    std::vector<MhdBlockView> v;
    v.reserve(blocks.size());
    for (const Block& b : blocks) v.push_back(b.fields);
    return v;
  }
  void check_(int rc) const {
    if (rc != MHD_OK) throw Error(rc, mhdvlct_last_error_string(h_));
  }
  mhdvlct_handle* h_ = nullptr;
};

}  // namespace mhdvlct

#endif  // MHDVLCT_METHOD_HPP
