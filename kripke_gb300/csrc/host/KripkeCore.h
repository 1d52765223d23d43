// KripkeCore.h -- RAJA-free Kripke data model over the kripke_gb300 C ABI.
//
// Mirrors the reference's Core layer (paths relative to the Kripke source tree):
//   Core::BaseVar / DataStore ...... src/Kripke/Core/BaseVar.h, Core/DataStore.h:23-89
//                                    (name -> variable; a missing name throws std::domain_error)
//   Core::Set (Range/GlobalRange) .. src/Kripke/Core/Set.h:23-202 (per-subdomain size and lower bound)
//   Core::Field .................... src/Kripke/Core/Field.h:29-290 (one chunk per subdomain of the
//                                    field's space, in the chosen nesting)
//   ArchLayoutV / layouts .......... src/Kripke/ArchLayout.h:32-147
//   InputVariables ................. src/Kripke/InputVariables.h:18-49
// A Field here is a handle on a device-resident field of the GB300 context: its
// host chunks are a mirror that is downloaded on first host access after the
// device changed it, and uploaded before the next kernel when the host changed
// it (the job CHAI does for the reference's CUDA build, without migrating every
// iteration).
#pragma once

#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "kgb.h"

namespace Kripke {

using SdomId = int;

enum ArchV { ArchV_Unknown = -1, ArchV_GB300 = 0, ArchV_num_values };
enum LayoutV { LayoutV_Unknown = -1, LayoutV_DGZ, LayoutV_DZG, LayoutV_GDZ, LayoutV_GZD, LayoutV_ZDG, LayoutV_ZGD, LayoutV_num_values };

std::string archToString(ArchV a);
ArchV stringToArch(const std::string &s);
std::string layoutToString(LayoutV l);
LayoutV stringToLayout(const std::string &s);

struct ArchLayoutV {
  ArchV arch_v;
  LayoutV layout_v;
};

enum ParallelMethod { PMETHOD_SWEEP, PMETHOD_BJ };

// InputVariables (src/Kripke/InputVariables.h:18-49) plus the generator and precision options.
struct InputVariables {
  InputVariables();
  bool checkValues() const;  // true on error (prints the reason)
  int nx, ny, nz;
  int num_directions, num_groups, legendre_order;
  int quad_num_polar, quad_num_azimuthal;
  ArchLayoutV al_v;
  int npx, npy, npz;
  int num_dirsets, num_groupsets;
  int num_zonesets_dim[3];
  int niter;
  ParallelMethod parallel_method;
  double sigt[3], sigs[3];
  int num_material_subsamples;
  std::string run_name;
  // additions: benchmark generator options and the precision form
  int geometry;    // 0 Kobayashi 3i, 1 100 cm cube
  int scatter;     // 0 diagonal P0, 1 seeded downscatter
  int perturb;     // seeded +-20% per (material, group)
  unsigned long long seed;
  int precision;   // KGB_FP64 or KGB_MIXED
  bool autotune;
  bool json;
};

namespace Core {

class BaseVar {
 public:
  virtual ~BaseVar() = default;
};

class DataStore {
 public:
  DataStore() = default;
  DataStore(const DataStore &) = delete;
  DataStore &operator=(const DataStore &) = delete;

  void addVariable(const std::string &name, BaseVar *var) {
    if (vars_.count(name)) throw std::domain_error("Variable '" + name + "' already exists");
    vars_[name].reset(var);
  }
  template <typename T, typename... A>
  T &newVariable(const std::string &name, A &&...args) {
    T *v = new T(std::forward<A>(args)...);
    addVariable(name, v);
    return *v;
  }
  void deleteVariable(const std::string &name) { vars_.erase(name); }
  template <typename T>
  T &getVariable(const std::string &name) {
    auto it = vars_.find(name);
    if (it == vars_.end()) throw std::domain_error("Cannot find '" + name + "' in DataStore");
    T *v = dynamic_cast<T *>(it->second.get());
    if (!v) throw std::domain_error("Variable '" + name + "' has a different type");
    return *v;
  }
  template <typename T>
  bool isVariableType(const std::string &name) const {
    auto it = vars_.find(name);
    return it != vars_.end() && dynamic_cast<T *>(it->second.get()) != nullptr;
  }
  std::vector<std::string> getVariableList() const {
    std::vector<std::string> n;
    for (auto &kv : vars_) n.push_back(kv.first);
    return n;
  }

 private:
  std::map<std::string, std::unique_ptr<BaseVar>> vars_;
};

// A set spanning subdomains: per-subdomain size and first global index.
class Set : public BaseVar {
 public:
  Set(std::vector<size_t> sizes, std::vector<size_t> lowers, size_t global)
      : size_(std::move(sizes)), lower_(std::move(lowers)), global_(global) {}
  size_t size(SdomId s) const { return size_.size() == 1 ? size_[0] : size_.at(s); }
  size_t lower(SdomId s) const { return lower_.size() == 1 ? lower_[0] : lower_.at(s); }
  size_t globalSize() const { return global_; }

 private:
  std::vector<size_t> size_, lower_;
  size_t global_;
};

// The GB300 context of a problem (DataStore name "gb300").
class Gb300Context : public BaseVar {
 public:
  explicit Gb300Context(int device);
  ~Gb300Context() override;
  kgb_ctx *ctx = nullptr;
  void check(int rc, const char *what) const;  // throws std::runtime_error on a failed call
};

// Handle on a device-resident field with a lazily synchronised host mirror
// (the concatenated chunks in the problem's nesting).
template <typename T>
class Field : public BaseVar {
 public:
  Field(Gb300Context &g, std::string name) : g_(&g), name_(std::move(name)) {}
  const std::string &name() const { return name_; }
  // host view of all chunks; downloads if the device copy is newer
  T *hostData() {
    if (!host_valid_) {
      int64_t nb = 0;
      g_->check(kgb_field_bytes(g_->ctx, name_.c_str(), &nb), "kgb_field_bytes");
      host_.resize((size_t)nb / sizeof(T));
      g_->check(kgb_field_download(g_->ctx, name_.c_str(), host_.data(), nb), "kgb_field_download");
      host_valid_ = true;
    }
    return host_.data();
  }
  size_t size() {
    hostData();
    return host_.size();
  }
  // after host writes: the next kernel sees them
  void markHostModified() {
    g_->check(kgb_field_upload(g_->ctx, name_.c_str(), host_.data(), (int64_t)(host_.size() * sizeof(T))),
              "kgb_field_upload");
  }
  // after a device write the mirror is stale
  void markDeviceModified() { host_valid_ = false; }
  Gb300Context &context() { return *g_; }

 private:
  Gb300Context *g_;
  std::string name_;
  std::vector<T> host_;
  bool host_valid_ = false;
};

}  // namespace Core

// Accumulating named wall-clock timers (src/Kripke/Timing.h:25-115).
class Timing : public Core::BaseVar {
 public:
  void start(const std::string &name);
  void stop(const std::string &name);
  void print() const;
  double getTotal(const std::string &name) const;
  size_t getCount(const std::string &name) const;

 private:
  struct T {
    double elapsed = 0.0, t0 = 0.0;
    size_t count = 0;
    bool running = false;
  };
  std::map<std::string, T> timers_;
};

class BlockTimer {
 public:
  BlockTimer(Timing &t, std::string n) : t_(t), n_(std::move(n)) { t_.start(n_); }
  ~BlockTimer() { t_.stop(n_); }

 private:
  Timing &t_;
  std::string n_;
};

#define KRIPKE_TIMER(DS, NAME) Kripke::BlockTimer BLK_TIMER_##NAME((DS).getVariable<Kripke::Timing>("timing"), #NAME)

class ArchLayout : public Core::BaseVar {
 public:
  ArchLayoutV al_v{ArchV_GB300, LayoutV_DGZ};
};

// Kripke::generateProblem (src/Kripke/Generate.cpp:24-94) on the GB300 path.
void generateProblem(Core::DataStore &ds, const InputVariables &vars);

// src/Kripke/Kernel.h:19-55
namespace Kernel {
void LPlusTimes(Core::DataStore &ds);
void LTimes(Core::DataStore &ds);
double population(Core::DataStore &ds);
void scattering(Core::DataStore &ds);
void source(Core::DataStore &ds);
void sweepSubdomain(Core::DataStore &ds, SdomId sdom_id);
void kConst(Core::Field<double> &field, double value);
}  // namespace Kernel

// Particle count after each source iteration, at full precision (the solver's
// printout keeps the reference's %e format).
struct ParticleHistory : public Core::BaseVar {
  std::vector<double> counts;
};

// src/Kripke/SweepSolver.h:20-22, SteadyStateSolver.h:18
void SweepSolver(Core::DataStore &ds, const std::vector<SdomId> &sdom_list, bool block_jacobi);
int SteadyStateSolver(Core::DataStore &ds, size_t max_iter, bool block_jacobi);

}  // namespace Kripke
