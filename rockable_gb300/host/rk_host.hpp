// rk_host.hpp -- C++ host of the GB300 engine: Rockable's input/output and
// plugin API around the C ABI of include/rk_gpu.h.
//
// The host keeps what Rockable's step loop keeps on the CPU -- the .conf
// keyword parser (src/Core/Rockable.cpp:643-1069), the shape library
// (src/Core/Shape.cpp:69-128), DrivingSystem (src/Core/DrivingSystem.cpp:44-268),
// conf writing (Rockable.cpp:440-610) and the ForceLaw / BodyForce /
// DataExtractor plugin registries -- and hands every step to the GPU engine
// through rk_step / rk_update_nl.  There is no CPU step.
#pragma once
#include <array>
#include <cstdint>
#include <fstream>
#include <functional>
#include <iosfwd>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/rk_gpu.h"

namespace rkhost {

class Rockable;

// ---------------------------------------------------------------- plugins --
// ForceLaw (src/ForceLaws/ForceLaw.hpp:44-55): init() registers the law's
// parameter names in the DataTable; the law itself runs on the GPU, selected
// by device_law().
class ForceLaw {
 public:
  Rockable* box{nullptr};
  virtual ~ForceLaw() = default;
  void plug(Rockable* b) { box = b; }
  virtual void init() = 0;
  virtual int device_law() const = 0;
};

// BodyForce (src/BodyForces/BodyForce.hpp:45-57).
class BodyForce {
 public:
  Rockable* box{nullptr};
  virtual ~BodyForce() = default;
  void plug(Rockable* b) { box = b; }
  virtual void read(std::istream& is) = 0;
  virtual void write(std::ostream& os) = 0;
  virtual void getForceAndMoment(size_t ibody, double force[3], double moment[3]) = 0;
  // the GPU step's form of the plugin: an RK_BF_* kind and the conf values
  // read() took, in that order (rk_set_body_force); -1 for a plugin that has
  // none (the step then refuses to run rather than evaluating it on the host)
  virtual int device_body_force(std::vector<double>& params) const { (void)params; return -1; }
};

// DataExtractor (src/DataExtractors/DataExtractor.hpp:46-73).  exec() and
// record() see the host mirror of the state, downloaded at their cadence
// (consoleRun: exec when step % nstep == 0, record when step % nrec == 0, with
// the reference's step counter, Rockable.cpp:2580, 2717-2738) -- except the
// extractors that reduce on the device (onDevice()): with a GPU context they
// read their few numbers through the rk_extract_* calls, and the mirror is
// not downloaded for them.
class DataExtractor {
 public:
  Rockable* box{nullptr};
  int nstep{1}, nrec{1};
  std::string filename;      // the data file, opened by read()
  std::ofstream recordFile;
  std::stringstream docString;
  std::vector<std::string> columnDoc;
  virtual ~DataExtractor() = default;
  void plug(Rockable* b) { box = b; }
  virtual void read(std::istream& is) = 0;
  virtual void init() {}
  virtual void exec() {}
  virtual void record() {}
  virtual void end() {}
  // record() reads the contact points of the entries (downloaded only on demand)
  virtual bool needsGeometry() const { return false; }
  // record() and exec() read the device, not the host mirror
  virtual bool onDevice() const { return false; }
  // the entry of extractedDataDoc.txt (DataExtractor.cpp: generateHelp)
  virtual void generateHelp(std::ostream& os);
};

template <class T>
class Factory {
 public:
  using Maker = std::function<T*()>;
  static Factory& instance() {
    static Factory f;
    return f;
  }
  void add(const std::string& name, Maker m) { makers_[name] = std::move(m); }
  T* create(const std::string& name) const {
    auto it = makers_.find(name);
    return it == makers_.end() ? nullptr : it->second();
  }

 private:
  std::map<std::string, Maker> makers_;
};

// --------------------------------------------------------------- state ----
struct Shape {  // Shape.hpp:58-111 (fields used by the step)
  std::string name;
  double radius{0.0}, volume{0.0};
  char preCompDone{'n'};
  double inertia_mass[3]{0, 0, 0};
  double obb[15]{0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0};  // center e1 e2 e3 extent
  std::vector<double> vertex;  // 3 per vertex
  std::vector<int> edge;       // 2 per edge
  std::vector<std::vector<int>> face;
};

struct Particles {  // SoA mirror of std::vector<Particle> (Particle.hpp:77-127)
  std::vector<int> shape, group, cluster;
  std::vector<double> homothety, mass, inertia, pos, vel, acc, Q, vrot, arot, force, moment;
  size_t size() const { return shape.size(); }
};

struct Interactions {  // key-sorted mirror of the neighbour list
  std::vector<int32_t> i, j, type, isub, jsub, bond;
  std::vector<double> n, dn, pos, vel, fn, ft, mom, damp;
  std::vector<uint8_t> active;
  size_t size() const { return i.size(); }
};

struct Interfaces {  // BreakableInterface.hpp:48-77
  std::vector<int32_t> i, j, nbonds, is_inner;
  std::vector<double> dn0, params;  // params: 8 per interface
  std::vector<std::vector<std::array<int32_t, 3>>> bonds;  // (type, isub, jsub)
  // per bond: 1 when it holds its interaction (stick set), 0 when the
  // interaction existed before stickVerticesInClusters made the bond: the
  // reference's set insert then keeps the old, unbonded interaction
  std::vector<std::vector<uint8_t>> live;
  std::vector<uint8_t> broken;
};

class Rockable {
 public:
  Rockable();
  ~Rockable();

  // I/O (Rockable.cpp:1085-1145, 440-610, 1187-1225)
  bool loadConf(const std::string& path);
  bool saveConf(const std::string& path);
  bool readDrivingSystem(const std::string& path);
  const std::string& error() const { return err_; }

  // the console run of src/Apps/run.cpp: initial NL update, integrate loop
  // writing conf<N> files into outdir; returns steps done or -1
  long consoleRun(const std::string& outdir, long max_steps = 0);
  // n passes of the integrate loop body without conf output
  bool run(long nsteps);
  bool updateNL();
  bool syncFromDevice(bool geometry);

  // options and state, named like the reference's members
  std::map<std::string, std::string> optionNames;
  double t{0.0}, tmax{1.0}, dt{1e-6}, interVerlet{0.01}, interConf{0.25}, DVerlet{0.0}, dVerlet{0.0};
  double gravity[3]{0.0, -9.81, 0.0};
  int paramsInInterfaces{0}, dynamicUpdateNL{0}, iconf{0}, precision{16};
  double dispUpdateNL{1.0}, angleUpdateNL{1.0}, numericalDampingCoeff{0.0};
  size_t nDriven{0};
  double cellMinSizes[3]{1, 1, 1};
  int boxForLinkCellsOpt{0};
  std::string shapeFile{"noShapeFile"}, parallel_mode{"DefaultParallelMode"};
  std::vector<Shape> Shapes;
  std::map<std::string, int> shapeId;
  Particles P;
  Interactions I;
  Interfaces F;
  std::map<int, double> density;
  // DataTable: parameter name -> (g1, g2) -> value
  std::map<std::string, std::map<std::pair<int, int>, double>> dataTable;
  std::unique_ptr<ForceLaw> forceLaw;
  std::unique_ptr<BodyForce> bodyForce;
  std::vector<std::unique_ptr<DataExtractor>> dataExtractors;
  std::vector<rk_control> controls;
  rk_servo servo{};
  double dataTableGet(const std::string& name, int g1, int g2) const;
  void dataTableSet(const std::string& name, int g1, int g2, double v);

  rk_ctx* ctx() { return ctx_; }

  // for the data extractors (Particle::GlobVertex / MinkowskiRadius,
  // Particle.cpp:55-71): vertex v of body b in world coordinates
  void globVertex(size_t b, size_t v, double out[3]) const;
  double minkowskiRadius(size_t b) const;
  // reads "name parameters" records from a dataExtractors.txt file
  // (Rockable::readDataExtractors, Rockable.cpp:1152-1180); unknown names are
  // reported and skipped; a missing file adds none
  bool readDataExtractors(const std::string& path);
  int computationStopAsked{0};  // set by an extractor: the run stops after one more step

 private:
  bool parse(std::istream& is);
  bool loadShapes(const std::string& path);
  bool upload();
  bool fail(const std::string& m) {
    err_ = m;
    return false;
  }
  bool ck(int rc, const char* what);
  void stickVerticesInClusters(double eps);
  void setVariableStickParams(const std::string& par, const std::string& io, double lambda, double m);
  std::string path_;
  std::string err_;
  rk_ctx* ctx_{nullptr};
  bool uploaded_{false};
  double interConfC_{0.0};
  long step_{0};
  bool extractorsRead_{false};
};

void register_builtin_plugins();
void register_builtin_extractors();  // rk_extractors.cpp

}  // namespace rkhost

extern "C" {
typedef struct rkh_sim rkh_sim;
rkh_sim* rkh_open(const char* conf_path);
const char* rkh_error(void);
void rkh_close(rkh_sim* s);
int rkh_read_driving(rkh_sim* s, const char* path);
long rkh_console_run(rkh_sim* s, const char* outdir, long max_steps);
int rkh_run(rkh_sim* s, long nsteps);
int rkh_save_conf(rkh_sim* s, const char* path);
/* The engine context the host drives (owned by the host: valid until
 * rkh_close), for direct rk_* calls on the loaded scene, e.g. rk_step. */
rk_ctx* rkh_context(rkh_sim* s);
}
