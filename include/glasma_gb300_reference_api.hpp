// glasma_gb300_reference_api.hpp -- C++ drop-in for the reference's hot-path call surface.
//
// The reference compiles its physics modules into its drivers as one translation unit
// (S/Simulation.cpp:6-103; S/ = the reference's SourceCode directory).  A driver written
// against that surface can include this header instead of the modules below and run the
// leapfrog, the observables and the gauge fixing on the GPU through include/glasma_gb300.h:
//
//   reference module                                   replaced by
//   S/LATTICE/GaugeLinks.cpp, ElectricFields.cpp,      GaugeLinks, ElectricFields, ChargeDensity,
//     ChargeDensity.cpp, GaugeTransformations.cpp        GaugeTransformations (same members)
//   S/LATTICE/SUNcVariables.cpp                        SUNcGaugeLinks::, SUNcElectricFields::,
//                                                        SUNcChargeDensity::, Lattice::Init
//   S/DYNAMICS/SUNcDynamics.cpp                        Dynamics::SUNc::Update and sub-steps
//   S/OBSERVABLES/BulkObservables.cpp                  Observables::Bulk
//   S/OBSERVABLES/GaussLawViolation.cpp                Observables::GaussLaw
//   S/OBSERVABLES/UnitarityViolation.cpp               Observables::Unitarity
//   S/OBSERVABLES/EnergyMomentumTensor.cpp             Observables::EnergyMomentumTensor::CreateMap
//   S/GAUGETRANSFORMATION/CoulombGaugeFixing.cpp       CoulombGaugeFixing::SetCoulombGauge
//
// Each container keeps a host mirror in the reference's layout (so Get(x,y,z,...) and
// SynchronizeGhostCells behave as before) and the lattice handle keeps the device copy.
// A field moves only when the other side needs it: host access through Get()/raw pointers
// marks the host copy as the newest, a GPU operation uploads such fields first and marks
// the fields it writes as newer on the device.  The evolve loop of the reference touches no
// field on the host between steps, so a run moves data only at initialisation and when the
// driver reads fields back.
//
// Errors: the reference calls exit(0) on numerical failure; here every failing library
// call throws glasma_dropin::Error carrying the status code.
#pragma once

#include <complex>
#include <cstring>
#include <fstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "glasma_gb300.h"

namespace glasma_dropin {

typedef double DOUBLE;
typedef int INT;
typedef std::complex<double> COMPLEX;

struct Error : std::runtime_error {
  int status;
  Error(int s, const std::string& m) : std::runtime_error(m), status(s) {}
};

inline void check(int status) {
  if (status != GLASMA_OK) throw Error(status, std::string(glasma_status_string(status)) + ": " + glasma_last_error());
}

// One GPU lattice shared by all containers of the same geometry (the reference's globals).
struct Device {
  glasma_lattice* h = nullptr;
  int N[3] = {0, 0, 0};
  static Device& get() {
    static Device d;
    return d;
  }
  void init(const int* n, const double* a, int precision = GLASMA_FP64, int reunitarize_every = 0) {
    if (h) glasma_destroy(h);
    check(glasma_create(n[0], n[1], n[2], a[0], a[1], a[2], precision, reunitarize_every, &h));
    for (int i = 0; i < 3; i++) N[i] = n[i];
  }
  ~Device() {
    if (h) glasma_destroy(h);
  }
};

// Host mirror of one device field.
class Mirror {
 public:
  enum State { kHostNewer, kDeviceNewer, kInSync };
  Mirror(int field, long long doubles) : field_(field), data_((size_t)doubles, 0.0), state_(kHostNewer) {}
  double* host_for_write() {
    pull();
    state_ = kHostNewer;
    return data_.data();
  }
  const double* host_for_read() {
    pull();
    return data_.data();
  }
  void push() {  // before a device operation reads the field
    if (state_ == kHostNewer) {
      check(glasma_upload(Device::get().h, field_, data_.data()));
      state_ = kInSync;
    }
  }
  void device_wrote() { state_ = kDeviceNewer; }
  int field() const { return field_; }

 private:
  void pull() {
    if (state_ == kDeviceNewer) {
      check(glasma_download(Device::get().h, field_, data_.data()));
      state_ = kInSync;
    }
  }
  int field_;
  std::vector<double> data_;
  State state_;
};

inline long long sites_with_ghosts(const int* N) { return (long long)N[0] * N[1] * (N[2] + 2); }

}  // namespace glasma_dropin

namespace Lattice {
static const int Dimension = 3;
inline glasma_dropin::INT N[3] = {128, 128, 2048};
inline glasma_dropin::DOUBLE a[3] = {1.0, 1.0, 0.25};
inline glasma_dropin::DOUBLE aScale = 1.0;
inline glasma_dropin::INT Volume = 0;
inline glasma_dropin::DOUBLE aCube = 0.0;
}  // namespace Lattice

// S/LATTICE/GaugeLinks.cpp:11-135
class GaugeLinks {
 public:
  glasma_dropin::INT Volume;
  static const glasma_dropin::INT Dimension = 3;
  glasma_dropin::DOUBLE a[Dimension];
  glasma_dropin::DOUBLE aCube;
  glasma_dropin::INT N[Dimension];
  glasma_dropin::Mirror mirror;

  GaugeLinks(int Nx, int Ny, int Nz, double ax, double ay, double az, int field = GLASMA_FIELD_U)
      : mirror(field, 54LL * Nx * Ny * (Nz + 2)) {
    N[0] = Nx; N[1] = Ny; N[2] = Nz;
    a[0] = ax; a[1] = ay; a[2] = az;
    Volume = Nx * Ny * Nz;
    aCube = ax * ay * az;
    SetIdentity();
  }
  long long Index3D(int x, int y, int z) const {
    const int xm = ((x % N[0]) + N[0]) % N[0], ym = ((y % N[1]) + N[1]) % N[1];
    return xm + (long long)N[0] * (ym + (long long)N[1] * (z + 1));
  }
  long long Index(int x, int y, int z, int mu) const { return 9 * (mu + 3 * Index3D(x, y, z)); }
  glasma_dropin::COMPLEX* Get(int x, int y, int z, int mu) {
    return reinterpret_cast<glasma_dropin::COMPLEX*>(mirror.host_for_write()) + Index(x, y, z, mu);
  }
  void SynchronizeGhostCells() {
    glasma_dropin::COMPLEX* U = reinterpret_cast<glasma_dropin::COMPLEX*>(mirror.host_for_write());
    const size_t n = 27 * (size_t)N[0] * N[1];
    std::memcpy(U + 27 * Index3D(0, 0, -1), U + 27 * Index3D(0, 0, 0), n * sizeof(glasma_dropin::COMPLEX));
    std::memcpy(U + 27 * Index3D(0, 0, N[2]), U + 27 * Index3D(0, 0, N[2] - 1), n * sizeof(glasma_dropin::COMPLEX));
  }
  void SetIdentity() {
    glasma_dropin::COMPLEX* U = reinterpret_cast<glasma_dropin::COMPLEX*>(mirror.host_for_write());
    const long long S = glasma_dropin::sites_with_ghosts(N);
    for (long long s = 0; s < S * 3; s++)
      for (int k = 0; k < 9; k++) U[9 * s + k] = (k % 4 == 0) ? 1.0 : 0.0;
  }
};

// S/LATTICE/ElectricFields.cpp:9-128
class ElectricFields {
 public:
  glasma_dropin::INT Volume;
  static const glasma_dropin::INT Dimension = 3;
  glasma_dropin::DOUBLE a[Dimension];
  glasma_dropin::DOUBLE aCube;
  glasma_dropin::INT N[Dimension];
  glasma_dropin::Mirror mirror;

  ElectricFields(int Nx, int Ny, int Nz, double ax, double ay, double az, int field = GLASMA_FIELD_E)
      : mirror(field, 24LL * Nx * Ny * (Nz + 2)) {
    N[0] = Nx; N[1] = Ny; N[2] = Nz;
    a[0] = ax; a[1] = ay; a[2] = az;
    Volume = Nx * Ny * Nz;
    aCube = ax * ay * az;
  }
  long long Index3D(int x, int y, int z) const {
    const int xm = ((x % N[0]) + N[0]) % N[0], ym = ((y % N[1]) + N[1]) % N[1];
    return xm + (long long)N[0] * (ym + (long long)N[1] * (z + 1));
  }
  long long Index(int x, int y, int z, int mu, int a_) const { return a_ + 8 * (mu + 3 * Index3D(x, y, z)); }
  double* Get(int x, int y, int z, int mu, int a_) { return mirror.host_for_write() + Index(x, y, z, mu, a_); }
  double GetValue(int x, int y, int z, int mu, int a_) { return mirror.host_for_read()[Index(x, y, z, mu, a_)]; }
  void SynchronizeGhostCells() {
    double* E = mirror.host_for_write();
    const size_t n = 24 * (size_t)N[0] * N[1];
    std::memcpy(E + 24 * Index3D(0, 0, -1), E + 24 * Index3D(0, 0, 0), n * sizeof(double));
    std::memcpy(E + 24 * Index3D(0, 0, N[2]), E + 24 * Index3D(0, 0, N[2] - 1), n * sizeof(double));
  }
  void SetZero() {
    double* E = mirror.host_for_write();
    std::memset(E, 0, sizeof(double) * 24 * glasma_dropin::sites_with_ghosts(N));
  }
};

// S/LATTICE/ChargeDensity.cpp:11-110
class ChargeDensity {
 public:
  glasma_dropin::INT Volume;
  static const glasma_dropin::INT Dimension = 3;
  glasma_dropin::DOUBLE a[Dimension];
  glasma_dropin::DOUBLE aCube;
  glasma_dropin::INT N[Dimension];
  glasma_dropin::Mirror mirror;

  ChargeDensity(int Nx, int Ny, int Nz, double ax, double ay, double az, int field)
      : mirror(field, 8LL * Nx * Ny * (Nz + 2)) {
    N[0] = Nx; N[1] = Ny; N[2] = Nz;
    a[0] = ax; a[1] = ay; a[2] = az;
    Volume = Nx * Ny * Nz;
    aCube = ax * ay * az;
  }
  long long Index3D(int x, int y, int z) const {
    const int xm = ((x % N[0]) + N[0]) % N[0], ym = ((y % N[1]) + N[1]) % N[1];
    return xm + (long long)N[0] * (ym + (long long)N[1] * (z + 1));
  }
  long long Index(int x, int y, int z, int a_) const { return a_ + 8 * Index3D(x, y, z); }
  double* Get(int x, int y, int z, int a_) { return mirror.host_for_write() + Index(x, y, z, a_); }
  double GetValue(int x, int y, int z, int a_) { return mirror.host_for_read()[Index(x, y, z, a_)]; }
  void SynchronizeGhostCells() {
    double* J = mirror.host_for_write();
    const size_t n = 8 * (size_t)N[0] * N[1];
    std::memcpy(J + 8 * Index3D(0, 0, -1), J + 8 * Index3D(0, 0, 0), n * sizeof(double));
    std::memcpy(J + 8 * Index3D(0, 0, N[2]), J + 8 * Index3D(0, 0, N[2] - 1), n * sizeof(double));
  }
  void SetZero() {
    double* J = mirror.host_for_write();
    std::memset(J, 0, sizeof(double) * 8 * glasma_dropin::sites_with_ghosts(N));
  }
};

// S/LATTICE/SUNcVariables.cpp:4-90: the global fields, allocated by Lattice::Init.
namespace SUNcGaugeLinks {
inline GaugeLinks *U = nullptr, *UOld = nullptr;
}
namespace SUNcElectricFields {
inline ElectricFields* E = nullptr;
}
namespace SUNcChargeDensity {
inline ChargeDensity *Jp = nullptr, *Jm = nullptr, *JpStat = nullptr, *JmStat = nullptr;
}

namespace Lattice {
inline void Init(int precision = GLASMA_FP64, int reunitarize_every = 0) {
  Volume = N[0] * N[1] * N[2];
  aCube = a[0] * a[1] * a[2];
  glasma_dropin::Device::get().init(N, a, precision, reunitarize_every);
  glasma_dropin::check(glasma_set_scale(glasma_dropin::Device::get().h, aScale));
  SUNcGaugeLinks::U = new GaugeLinks(N[0], N[1], N[2], a[0], a[1], a[2], GLASMA_FIELD_U);
  SUNcGaugeLinks::UOld = new GaugeLinks(N[0], N[1], N[2], a[0], a[1], a[2], GLASMA_FIELD_UOLD);
  SUNcElectricFields::E = new ElectricFields(N[0], N[1], N[2], a[0], a[1], a[2], GLASMA_FIELD_E);
  SUNcChargeDensity::Jp = new ChargeDensity(N[0], N[1], N[2], a[0], a[1], a[2], GLASMA_FIELD_JP);
  SUNcChargeDensity::Jm = new ChargeDensity(N[0], N[1], N[2], a[0], a[1], a[2], GLASMA_FIELD_JM);
  SUNcChargeDensity::JpStat = new ChargeDensity(N[0], N[1], N[2], a[0], a[1], a[2], GLASMA_FIELD_JPSTAT);
  SUNcChargeDensity::JmStat = new ChargeDensity(N[0], N[1], N[2], a[0], a[1], a[2], GLASMA_FIELD_JMSTAT);
}
}  // namespace Lattice

namespace glasma_dropin {
inline glasma_lattice* handle() { return Device::get().h; }
template <typename... F>
inline void push(F*... f) {
  (f->mirror.push(), ...);
}
template <typename... F>
inline void wrote(F*... f) {
  (f->mirror.device_wrote(), ...);
}
}  // namespace glasma_dropin

// S/DYNAMICS/SUNcDynamics.cpp
namespace Dynamics {
inline glasma_dropin::DOUBLE t = 0.0, t0 = 0.0, dTStep = 0.08;
inline glasma_dropin::INT tSteps = 0;
inline glasma_dropin::DOUBLE Time() { return t; }
inline void Reset() {
  t = t0;
  tSteps = 0;
}
namespace SUNc {
// The containers passed in must be the global ones Lattice::Init created (the device holds one lattice).
inline void Update(GaugeLinks* U, ElectricFields* E, ChargeDensity* Jp, ChargeDensity* Jm, ChargeDensity* JpStat,
                   ChargeDensity* JmStat) {
  glasma_dropin::push(U, E, Jp, Jm, JpStat, JmStat);
  glasma_dropin::check(glasma_step(glasma_dropin::handle(), dTStep, 1, GLASMA_STEP_SAVE_UOLD));
  glasma_dropin::wrote(U, E, Jp, Jm, JpStat, JmStat, SUNcGaugeLinks::UOld);
  tSteps++;
  t += dTStep;
}
inline void UpdateElectricFields(GaugeLinks* U, ElectricFields* E, ChargeDensity* Jp, ChargeDensity* Jm, double dt) {
  glasma_dropin::push(U, E, Jp, Jm);
  glasma_dropin::check(glasma_update_efield(glasma_dropin::handle(), dt));
  glasma_dropin::wrote(U, E);
}
inline void UpdateGaugeLinks(GaugeLinks* U, ElectricFields* E, double dt_arg) {
  glasma_dropin::push(U, E);
  glasma_dropin::check(glasma_update_links(glasma_dropin::handle(), dt_arg));
  glasma_dropin::wrote(U);
}
}  // namespace SUNc
}  // namespace Dynamics

// S/OBSERVABLES/BulkObservables.cpp:4-191
namespace Observables {
namespace Bulk {
inline glasma_dropin::DOUBLE ESqr[3], BSqr[3], EDotJ[3];
inline glasma_dropin::DOUBLE out_[16];
inline void Update(GaugeLinks* U, ElectricFields* E, ChargeDensity* Jp, ChargeDensity* Jm) {
  glasma_dropin::push(U, E, Jp, Jm);
  glasma_dropin::check(glasma_bulk(glasma_dropin::handle(), out_));
  for (int i = 0; i < 3; i++) {
    ESqr[i] = out_[i];
    BSqr[i] = out_[3 + i];
    EDotJ[i] = out_[6 + i];
  }
}
inline void Update() { Update(SUNcGaugeLinks::U, SUNcElectricFields::E, SUNcChargeDensity::Jp, SUNcChargeDensity::Jm); }
inline glasma_dropin::DOUBLE T00() { return out_[9]; }
inline glasma_dropin::DOUBLE TXX() { return out_[10]; }
inline glasma_dropin::DOUBLE TYY() { return out_[11]; }
inline glasma_dropin::DOUBLE TZZ() { return out_[12]; }
inline glasma_dropin::DOUBLE ELECTRIC() { return out_[13]; }
inline glasma_dropin::DOUBLE MAGNETIC() { return out_[14]; }
inline glasma_dropin::DOUBLE SOURCE() { return out_[15]; }
}  // namespace Bulk

// S/OBSERVABLES/GaussLawViolation.cpp:4-165
namespace GaussLaw {
inline glasma_dropin::DOUBLE GlobalMaxViolation = 0.0, GlobalAvgViolation = 0.0;
inline void UpdateViolation(GaugeLinks* U, ElectricFields* E, ChargeDensity* JpStat, ChargeDensity* JmStat) {
  glasma_dropin::push(U, E, JpStat, JmStat);
  glasma_dropin::check(glasma_gauss(glasma_dropin::handle(), 0, &GlobalMaxViolation, &GlobalAvgViolation, nullptr));
}
// Per-z form: syncs the ghosts first and writes "z  sum_{x,y,a} G^2/(Nx Ny)" lines to fname.
inline void UpdateViolation(GaugeLinks* U, ElectricFields* E, ChargeDensity* JpStat, ChargeDensity* JmStat,
                            const std::string& fname) {
  glasma_dropin::push(U, E, JpStat, JmStat);
  std::vector<double> prof((size_t)Lattice::N[2]);
  glasma_dropin::check(glasma_gauss(glasma_dropin::handle(), 1, &GlobalMaxViolation, &GlobalAvgViolation, prof.data()));
  glasma_dropin::wrote(U, E, JpStat, JmStat);  // ghost slices were synced on the device
  std::ofstream out(fname.c_str());
  out.precision(15);
  for (size_t z = 0; z < prof.size(); z++) out << z << "  " << prof[z] << "\n";
}
}  // namespace GaussLaw

// S/OBSERVABLES/UnitarityViolation.cpp:4-69
namespace Unitarity {
inline glasma_dropin::DOUBLE GlobalMaxViolation = 0.0, GlobalAvgViolation = 0.0;
inline void UpdateViolation(GaugeLinks* U) {
  glasma_dropin::push(U);
  glasma_dropin::check(glasma_unitarity(glasma_dropin::handle(), &GlobalMaxViolation, &GlobalAvgViolation));
}
inline void CheckViolation() { UpdateViolation(SUNcGaugeLinks::U); }
}  // namespace Unitarity

// S/OBSERVABLES/EnergyMomentumTensor.cpp:92-184: writes "z T00 TXX TYY TZZ T0X T0Y T0Z TXY TYZ TZX" lines.
namespace EnergyMomentumTensor {
inline std::vector<double> Map;
inline void CreateMap(const std::string& fname, GaugeLinks* U, GaugeLinks* UOld, ElectricFields* E) {
  glasma_dropin::push(U, UOld, E);
  Map.assign((size_t)Lattice::N[2] * 10, 0.0);
  glasma_dropin::check(glasma_emt_map(glasma_dropin::handle(), Map.data()));
  glasma_dropin::wrote(U, UOld);  // ghost slices synced on the device
  if (fname.empty()) return;
  std::ofstream out(fname.c_str());
  out.precision(15);
  for (int z = 0; z < Lattice::N[2]; z++) {
    out << z;
    for (int k = 0; k < 10; k++) out << "  " << Map[(size_t)z * 10 + k];
    out << "\n";
  }
}
}  // namespace EnergyMomentumTensor
}  // namespace Observables

// S/IO/SaveConfiguration.cpp:6-93 and S/IO/LoadConfiguration.cpp:3-200: text configuration files,
// named as the reference names them (OutputDirectory + stem + "ID" + seed + ".txt").  Errors throw
// glasma_dropin::Error where the reference exits.
namespace RandomNumberGenerator {
inline long int MySEED = 0;
}
namespace IO {
inline std::string OutputDirectory = "";
inline std::string ConfigurationFileName(const std::string& stem) {
  return OutputDirectory + stem + "ID" + std::to_string(RandomNumberGenerator::MySEED) + ".txt";
}
inline void io_check(int status) {
  if (status != GLASMA_OK)
    throw glasma_dropin::Error(status, std::string(glasma_status_string(status)) + ": " + glasma_io_last_error());
}
inline void SaveConfiguration(const std::string& Ufname, const std::string& Efname) {
  glasma_dropin::push(SUNcGaugeLinks::U, SUNcElectricFields::E);
  io_check(glasma_save_text(glasma_dropin::handle(), ConfigurationFileName(Ufname).c_str(),
                            ConfigurationFileName(Efname).c_str(), nullptr));
}
inline void SaveConfigurationJ(const std::string& Jfname) {
  glasma_dropin::push(SUNcChargeDensity::Jp, SUNcChargeDensity::Jm, SUNcChargeDensity::JpStat,
                      SUNcChargeDensity::JmStat);
  io_check(glasma_save_text(glasma_dropin::handle(), nullptr, nullptr, ConfigurationFileName(Jfname).c_str()));
}
// Full paths, as the reference's loader takes them.
inline void LoadConfiguration(const std::string& Ufname, const std::string& Efname, const std::string& Jfname) {
  io_check(glasma_load_text(glasma_dropin::handle(), Ufname.c_str(), Efname.c_str(), Jfname.c_str()));
  glasma_dropin::wrote(SUNcGaugeLinks::U, SUNcElectricFields::E, SUNcChargeDensity::Jp, SUNcChargeDensity::Jm,
                       SUNcChargeDensity::JpStat, SUNcChargeDensity::JmStat);
}
}  // namespace IO

// S/GAUGETRANSFORMATION/CoulombGaugeFixing.cpp:6-96.  The reference compiles one of its three updates,
// chosen by a #define in CoulombGaugeFixing.cpp:4; here the same macro names, defined before this header
// is included, choose it (GAUGE_FIXING_ALGORITHM_LOS_ALAMOS, GAUGE_FIXING_ALGORITHM_JACOBI), and the
// Fourier-accelerated update is the default, as in the reference.  Defining GAUGE_FIXING_OPEN_Z as well
// selects the open-z functional for the Fourier update (GLASMA_GF_OPEN_Z: the top slice's z link into
// the ghost slice left out of the deviation), with which the iteration converges on open-z lattices
// where the reference's leaves SU(3); Flags can also be set at run time (GLASMA_GF_MIXED adds FP32
// sweeps before the final FP64 ones).
namespace CoulombGaugeFixing {
#if defined(GAUGE_FIXING_OPEN_Z)
inline unsigned Flags = GLASMA_GF_OPEN_Z;
#else
inline unsigned Flags = 0;  // glasma_coulomb_fix flags for the Fourier update
#endif
inline glasma_dropin::DOUBLE GlobalMaxDeviation = 0.0, GlobalAvgDeviation = 0.0, GlobalMaxStepSize = 0.0,
                             GlobalAvgStepSize = 0.0, GlobalMinGaugeFunctional = 0.0, GlobalSumGaugeFunctional = 0.0;
namespace FourierAccelerationAlgorithm {
inline glasma_dropin::DOUBLE alphaStepSize = 2.0;  // FourierAcceleration.cpp:6
}
namespace LosAlamosAlgorithm {
inline glasma_dropin::DOUBLE OverRelaxationProbability = 0.0;  // LosAlamos.cpp:6
// the over-relaxation draws: a counter-based hash of (DrawSeed, iteration, pass, site)
inline unsigned long long DrawSeed = 0;
}
namespace JacobiAlgorithm {
inline glasma_dropin::DOUBLE alphaStepSize = 0.3;  // Jacobi.cpp:6
}
// Writes one log line per iteration to fname (n, max dev, avg dev, max step, avg step, min F, sum F / V).
inline void SetCoulombGauge(const std::string& fname, int TotalSteps) {
  glasma_dropin::push(SUNcGaugeLinks::U, SUNcElectricFields::E);
  std::vector<double> log((size_t)(TotalSteps > 0 ? TotalSteps : 1) * 7);
  int n = 0;
#if defined(GAUGE_FIXING_ALGORITHM_LOS_ALAMOS)
  const int algorithm = GLASMA_GF_LOS_ALAMOS;
  const double param = LosAlamosAlgorithm::OverRelaxationProbability;
#elif defined(GAUGE_FIXING_ALGORITHM_JACOBI)
  const int algorithm = GLASMA_GF_JACOBI;
  const double param = JacobiAlgorithm::alphaStepSize;
#else
  const int algorithm = GLASMA_GF_FOURIER;
  const double param = FourierAccelerationAlgorithm::alphaStepSize;
#endif
  glasma_dropin::check(glasma_coulomb_fix_algorithm(glasma_dropin::handle(), algorithm, param,
                                                    LosAlamosAlgorithm::DrawSeed, TotalSteps, 1e-15,
                                                    algorithm == GLASMA_GF_FOURIER ? Flags : 0u, log.data(), &n));
  if (n > 0) {
    const double* last = log.data() + (size_t)(n - 1) * 7;
    GlobalMaxDeviation = last[1];
    GlobalAvgDeviation = last[2];
    GlobalMaxStepSize = last[3];
    GlobalAvgStepSize = last[4];
    GlobalMinGaugeFunctional = last[5];
    GlobalSumGaugeFunctional = last[6];
  }
  if (fname.empty()) return;
  std::ofstream out(fname.c_str());
  for (int i = 0; i < n; i++) {
    for (int k = 0; k < 7; k++) out << (k ? " " : "") << log[(size_t)i * 7 + k];
    out << "\n";
  }
}
inline void SetCoulombGauge(const std::string& fname) { SetCoulombGauge(fname, 1000); }
}  // namespace CoulombGaugeFixing
