/* Stand-ins for Cello's Block / Field / Data, exposing only what the VL+CT
 * toolkit touches: block->data()->field().view<T>(name). */
#ifndef ORACLE_SHIM_MESH_HPP
#define ORACLE_SHIM_MESH_HPP
#include <map>
#include <string>
enum class ghost_choice { include, exclude, permit };
enum precision_type { precision_unknown, precision_default, precision_single,
                      precision_double, precision_extended80,
                      precision_extended96, precision_quadruple };
class Field {
 public:
  template <class T> CelloView<T, 3> view(const std::string& name,
                                          ghost_choice, int) const {
    return views->at(name);
  }
  int precision(int) const { return precision_default; }
  void* values(const std::string&, int = 0) const { return nullptr; }
  bool ghosts_allocated() const { return true; }
  double history_time(int) const { return 0.0; }
  void ghost_depth(int, int* gx, int* gy, int* gz) const {
    if (gx) *gx = 0; if (gy) *gy = 0; if (gz) *gz = 0;
  }
  void size(int* nx, int* ny, int* nz) const {
    if (nx) *nx = 0; if (ny) *ny = 0; if (nz) *nz = 0;
  }
  void* values(int, int = 0) const { return nullptr; }
  std::map<std::string, CelloView<double, 3>>* views = nullptr;
  template <class T> CelloView<T, 3> view(const std::string& name) const {
    return views->at(name);
  }
  int field_id(const std::string& name) const {
    return views->count(name) ? 0 : -1;
  }
  bool is_field(const std::string& name) const { return views->count(name) > 0; }
};
class Data {
 public:
  Field field_;
  Field field() { return field_; }
};
class Block {
 public:
  Data data_;
  Data* data() { return &data_; }
  void cell_width(double* hx, double* hy, double* hz) const {
    *hx = *hy = *hz = 1.0;
  }
  virtual ~Block() {}
  bool is_leaf() const { return true; }
  double time() const { return 0.0; }
  std::string name() const { return "block"; }
};
class FieldDescr {
 public:
  bool is_field(const std::string&) const { return true; }
  int field_id(const std::string&) const { return 0; }
  void centering(int, int* cx, int* cy, int* cz) const {
    *cx = *cy = *cz = 0;
  }
};
namespace cello {
FieldDescr* field_descr();
}
class Physics {
 public:
  Physics() {}
  Physics(CkMigrateMessage*) {}
  virtual ~Physics() {}
  virtual std::string type() const = 0;
  virtual void pup(PUP::er&) {}
};
class Compute {
 public:
  Compute() {}
  Compute(CkMigrateMessage*) {}
  virtual ~Compute() {}
  virtual void pup(PUP::er&) {}
  int i_hist_ = 0;
};
#endif
