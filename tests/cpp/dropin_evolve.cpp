// A driver written against the reference's call surface (as S/Simulation.cpp:212-321 uses it),
// compiled against include/glasma_gb300_reference_api.hpp instead of the reference's modules.
// Usage: dropin_evolve Nx Ny Nz dt nsteps in_prefix out_prefix
// Reads <in_prefix>.{U,E,Jp,Jm,JpStat,JmStat}.bin (reference host layout, FP64), evolves, writes
// <out_prefix>.{U,UOld,E,Jp,Jm,JpStat,JmStat}.bin, the reference's text configuration files
// <out_prefix>.{U,E,J}ID<seed>.txt (IO::SaveConfiguration / SaveConfigurationJ) and prints the bulk
// energy and Gauss law.
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <string>
#include <vector>

#include "glasma_gb300_reference_api.hpp"

static void read_into(const std::string& path, double* dst, size_t n) {
  std::ifstream in(path, std::ios::binary);
  in.read(reinterpret_cast<char*>(dst), n * sizeof(double));
  if (!in) {
    std::fprintf(stderr, "cannot read %s\n", path.c_str());
    std::exit(2);
  }
}
static void write_from(const std::string& path, const double* src, size_t n) {
  std::ofstream out(path, std::ios::binary);
  out.write(reinterpret_cast<const char*>(src), n * sizeof(double));
}

int main(int argc, char** argv) {
  if (argc != 8) return 2;
  Lattice::N[0] = std::atoi(argv[1]);
  Lattice::N[1] = std::atoi(argv[2]);
  Lattice::N[2] = std::atoi(argv[3]);
  Lattice::a[0] = Lattice::a[1] = Lattice::a[2] = 1.0;
  Dynamics::dTStep = std::atof(argv[4]);
  const int nsteps = std::atoi(argv[5]);
  const std::string in = argv[6], out = argv[7];
  try {
    Lattice::Init();
    const size_t S = (size_t)Lattice::N[0] * Lattice::N[1] * (Lattice::N[2] + 2);
    // host-side initial conditions written through the containers, as the reference's initial-condition code does
    read_into(in + ".U.bin", reinterpret_cast<double*>(SUNcGaugeLinks::U->Get(0, 0, -1, 0)), 54 * S);
    read_into(in + ".E.bin", SUNcElectricFields::E->Get(0, 0, -1, 0, 0), 24 * S);
    read_into(in + ".Jp.bin", SUNcChargeDensity::Jp->Get(0, 0, -1, 0), 8 * S);
    read_into(in + ".Jm.bin", SUNcChargeDensity::Jm->Get(0, 0, -1, 0), 8 * S);
    read_into(in + ".JpStat.bin", SUNcChargeDensity::JpStat->Get(0, 0, -1, 0), 8 * S);
    read_into(in + ".JmStat.bin", SUNcChargeDensity::JmStat->Get(0, 0, -1, 0), 8 * S);
    Dynamics::Reset();
    for (int n = 0; n < nsteps; n++)
      Dynamics::SUNc::Update(SUNcGaugeLinks::U, SUNcElectricFields::E, SUNcChargeDensity::Jp, SUNcChargeDensity::Jm,
                             SUNcChargeDensity::JpStat, SUNcChargeDensity::JmStat);
    Observables::Bulk::Update();
    Observables::GaussLaw::UpdateViolation(SUNcGaugeLinks::U, SUNcElectricFields::E, SUNcChargeDensity::JpStat,
                                           SUNcChargeDensity::JmStat);
    std::printf("T00 %.17g\nSOURCE %.17g\nGAUSS %.17g %.17g\nTIME %.17g\n", Observables::Bulk::T00(),
                Observables::Bulk::SOURCE(), Observables::GaussLaw::GlobalMaxViolation,
                Observables::GaussLaw::GlobalAvgViolation, Dynamics::Time());
    write_from(out + ".U.bin", reinterpret_cast<double*>(SUNcGaugeLinks::U->Get(0, 0, -1, 0)), 54 * S);
    write_from(out + ".UOld.bin", reinterpret_cast<double*>(SUNcGaugeLinks::UOld->Get(0, 0, -1, 0)), 54 * S);
    write_from(out + ".E.bin", SUNcElectricFields::E->Get(0, 0, -1, 0, 0), 24 * S);
    write_from(out + ".Jp.bin", SUNcChargeDensity::Jp->Get(0, 0, -1, 0), 8 * S);
    write_from(out + ".Jm.bin", SUNcChargeDensity::Jm->Get(0, 0, -1, 0), 8 * S);
    write_from(out + ".JpStat.bin", SUNcChargeDensity::JpStat->Get(0, 0, -1, 0), 8 * S);
    write_from(out + ".JmStat.bin", SUNcChargeDensity::JmStat->Get(0, 0, -1, 0), 8 * S);
    IO::OutputDirectory = out + ".";
    IO::SaveConfiguration("U", "E");
    IO::SaveConfigurationJ("J");
  } catch (const glasma_dropin::Error& e) {
    std::fprintf(stderr, "glasma error %d: %s\n", e.status, e.what());
    return 3;
  }
  return 0;
}
