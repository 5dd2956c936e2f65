// ref_harness.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Compiles the reference's own SU(3) code path from its unmodified source files
// (included from the reference checkout, which is passed with -I) into a shared
// library with a small C interface, so that the oracle restatement and the
// golden fixtures can be pinned against the reference itself.
//
// What this file adds, and nothing else:
//   * M_SQRT3, and SU(3) AdjointMultiplication / InverseAdjointMultiplication /
//     MatrixILog, which the reference only defines for SU(2) and U(1)
//     (S/SUNc/SU2/AlgebraOperations.cpp:90-124, S/SUNc/U1/AlgebraOperations.cpp:41-46);
//   * a RandomNumberGenerator namespace that replays injected Gaussian numbers in
//     place of S/MISC/RNG/GSLRandomNumberGenerator.cpp (GSL is not installed);
//   * the fftw3.h stand-in next to this file (FFTW is not installed);
//   * extern "C" accessors.  The driver files (S/Simulation.cpp etc.) are not
//     compiled; their include order (S/Simulation.cpp:6-103) is followed.
#include "Definitions.cpp"

#define SU_Nc_FLAG SU3_FLAG
#ifndef M_SQRT3
#define M_SQRT3 1.73205080756887729352744634150587236694280525381038
#endif

#include "SUNc/Definitions.cpp"

// ---- SU(3) pieces the reference leaves undefined -------------------------------
namespace SUNcAlgebra {
namespace Operations {

static void HarnessHermFromAlgebra(const SU_Nc_ALGEBRA_FORMAT* e, SU_Nc_FUNDAMENTAL_FORMAT* M) {
  COMPLEX A[3][3];
  MatrixForm(const_cast<SU_Nc_ALGEBRA_FORMAT*>(e), A);
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) M[SUNcGroup::MatrixIndex(i, j)] = A[i][j];
}
// out^a = 2 tr(t^a W), W Hermitian
static void HarnessAlgebraFromHerm(const SU_Nc_FUNDAMENTAL_FORMAT* W, SU_Nc_ALGEBRA_FORMAT* out) {
  using SUNcGroup::MatrixIndex;
  out[0] = 2.0 * real(W[MatrixIndex(0, 1)]);
  out[1] = -2.0 * imag(W[MatrixIndex(0, 1)]);
  out[2] = real(W[MatrixIndex(0, 0)]) - real(W[MatrixIndex(1, 1)]);
  out[3] = 2.0 * real(W[MatrixIndex(0, 2)]);
  out[4] = -2.0 * imag(W[MatrixIndex(0, 2)]);
  out[5] = 2.0 * real(W[MatrixIndex(1, 2)]);
  out[6] = -2.0 * imag(W[MatrixIndex(1, 2)]);
  out[7] = (real(W[MatrixIndex(0, 0)]) + real(W[MatrixIndex(1, 1)]) - 2.0 * real(W[MatrixIndex(2, 2)])) / M_SQRT3;
}

// V (t.E) V^dagger
void AdjointMultiplication(SU_Nc_FUNDAMENTAL_FORMAT* V, SU_Nc_ALGEBRA_FORMAT* E, SU_Nc_ALGEBRA_FORMAT* ENew) {
  SU_Nc_FUNDAMENTAL_FORMAT M[9], T[9], W[9];
  HarnessHermFromAlgebra(E, M);
  SUNcGroup::Operations::UU(V, M, T);
  SUNcGroup::Operations::UD(T, V, W);
  HarnessAlgebraFromHerm(W, ENew);
}
// V^dagger (t.E) V
void InverseAdjointMultiplication(SU_Nc_FUNDAMENTAL_FORMAT* V, SU_Nc_ALGEBRA_FORMAT* E, SU_Nc_ALGEBRA_FORMAT* ENew) {
  SU_Nc_FUNDAMENTAL_FORMAT M[9], T[9], W[9];
  HarnessHermFromAlgebra(E, M);
  SUNcGroup::Operations::DU(V, M, T);
  SUNcGroup::Operations::UU(T, V, W);
  HarnessAlgebraFromHerm(W, ENew);
}
// Solves exp(i C t^a L^a) = W for W in SU(3) near the identity: start from the
// anti-Hermitian part, then refine L <- L + P[(R - R^dagger)/2i], R = exp(-i L) W,
// P the traceless projection (twelve sweeps; the error shrinks by ~|L|/2 per sweep).
void MatrixILog(DOUBLE C, SU_Nc_FUNDAMENTAL_FORMAT* W, DOUBLE* LogW) {
  using SUNcGroup::MatrixIndex;
  SU_Nc_FUNDAMENTAL_FORMAT H[9];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      H[MatrixIndex(i, j)] = (W[MatrixIndex(i, j)] - conj(W[MatrixIndex(j, i)])) / COMPLEX(0.0, 2.0);
  DOUBLE L[8];
  HarnessAlgebraFromHerm(H, L);
  for (int it = 0; it < 12; it++) {
    SU_Nc_FUNDAMENTAL_FORMAT R0[9], R[9];
    MatrixIExp(-1.0, L, R0);
    SUNcGroup::Operations::UU(R0, W, R);
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++)
        H[MatrixIndex(i, j)] = (R[MatrixIndex(i, j)] - conj(R[MatrixIndex(j, i)])) / COMPLEX(0.0, 2.0);
    DOUBLE d[8];
    HarnessAlgebraFromHerm(H, d);
    for (int a = 0; a < 8; a++) L[a] += d[a];
  }
  for (int a = 0; a < 8; a++) LogW[a] = L[a] / C;
}

}  // namespace Operations
}  // namespace SUNcAlgebra

// ---- injected random numbers (replaces the GSL generator) ----------------------
namespace RandomNumberGenerator {
long int MySEED = 0;
static std::vector<double> Injected;
static size_t Cursor = 0;
void Init(long int SEED) { MySEED = SEED; }
DOUBLE Gauss() { return Cursor < Injected.size() ? Injected[Cursor++] : 0.0; }
// rng() replays injected uniforms (the Los Alamos over-relaxation draws), 0.5 once they run out
static std::vector<double> Uniforms;
static size_t UniformCursor = 0;
DOUBLE rng() { return UniformCursor < Uniforms.size() ? Uniforms[UniformCursor++] : 0.5; }
std::complex<DOUBLE> ComplexGauss() {
  DOUBLE re = Gauss(), im = Gauss();
  return std::complex<DOUBLE>(re, im) / M_SQRT2;
}
void SUNcMatrix(DOUBLE Amplitude, SU_Nc_FUNDAMENTAL_FORMAT* V) {
  SU_Nc_ALGEBRA_FORMAT alpha[SUNcAlgebra::NumberOfGenerators];
  for (int a = 0; a < SUNcAlgebra::NumberOfGenerators; a++) alpha[a] = rng();
  SUNcAlgebra::Operations::MatrixIExp(Amplitude, alpha, V);
}
}  // namespace RandomNumberGenerator

#include "LATTICE/3DGrid.cpp"
#include "LATTICE/Parameters.cpp"
#include "LATTICE/WilsonLines.cpp"
#include "LATTICE/GaugeLinks.cpp"
#include "LATTICE/ElectricFields.cpp"
#include "LATTICE/GaugeTransformations.cpp"
#include "LATTICE/ChargeDensity.cpp"
#include "LATTICE/SUNcVariables.cpp"
#include "LATTICE/Indexing.cpp"
#include "LATTICE/FourierSpace.cpp"
#include "CALC/Plaquettes.cpp"
#include "CALC/AvgFieldStrength.cpp"
#include "CALC/GaussViolation.cpp"
#include "CALC/GaugeTransformation.cpp"
#include "SUNcIndexing.cpp"
#include "IO/StringManipulation.cpp"
#include "IO/OutputManagement.cpp"
#include "DYNAMICS/SUNcDynamics.cpp"
#include "OBSERVABLES/BulkObservables.cpp"
#include "OBSERVABLES/GaussLawViolation.cpp"
#include "OBSERVABLES/UnitarityViolation.cpp"
#include "OBSERVABLES/EnergyMomentumTensor.cpp"
#include "GAUGETRANSFORMATION/GaugeTransformation.cpp"
#include "GAUGETRANSFORMATION/CoulombGaugeFixing.cpp"
#include "FFT/FFT1D.cpp"
#include "FFT/FFT2D.cpp"
#include "FFT/FFT3D.cpp"
#include "COLLIDINGOBJECTS/CollidingObjects.cpp"
#include "TMDNUCLEUS/NuclearData.cpp"
#include "TMDNUCLEUS/GBWSampling.cpp"
#include "TMDNUCLEUS/CorrelationFunction.cpp"
#include "TMDNUCLEUS/TMDbased.cpp"
#include "INITIALCONDITIONS/SUNCCURRENTS/RevSingleNucleus.cpp"
#include "IO/SaveConfiguration.cpp"
#include "IO/LoadConfiguration.cpp"

#include <cstdio>
#include <fstream>
#include <sstream>

// ---- C interface -------------------------------------------------------------
namespace {
bool g_ready = false;
std::string g_outdir = "/tmp";

long SitesWithGhosts() { return (long)Lattice::N[0] * Lattice::N[1] * (Lattice::N[2] + 2); }

void* FieldPointer(int which, long* n_doubles) {
  const long S = SitesWithGhosts();
  switch (which) {
    case 0: *n_doubles = 2 * 27 * S; return SUNcGaugeLinks::U->U;
    case 1: *n_doubles = 2 * 27 * S; return SUNcGaugeLinks::UOld->U;
    case 2: *n_doubles = 24 * S; return SUNcElectricFields::E->E;
    case 3: *n_doubles = 8 * S; return SUNcChargeDensity::Jp->J;
    case 4: *n_doubles = 8 * S; return SUNcChargeDensity::Jm->J;
    case 5: *n_doubles = 8 * S; return SUNcChargeDensity::JpStat->J;
    case 6: *n_doubles = 8 * S; return SUNcChargeDensity::JmStat->J;
    case 7: *n_doubles = 2 * 9 * S; return GaugeTransformation::G->G;
    case 8: *n_doubles = 2 * 27 * S; return GaugeFixedVariables::U->U;
    case 9: *n_doubles = 24 * S; return GaugeFixedVariables::E->E;
    // the initial-condition intermediates (S/LATTICE/SUNcVariables.cpp:41-60)
    case 10: *n_doubles = 8 * S; return SUNcChargeDensity::rhoL->J;
    case 11: *n_doubles = 8 * S; return SUNcChargeDensity::rhoR->J;
    case 12: *n_doubles = 8 * S; return SUNcChargeDensity::CFL->J;
    case 13: *n_doubles = 8 * S; return SUNcChargeDensity::CFR->J;
    case 14: *n_doubles = 8 * S; return SUNcChargeDensity::RhoLT1->J;
    case 15: *n_doubles = 8 * S; return SUNcChargeDensity::RhoRT1->J;
    case 16: *n_doubles = 2 * 9 * S; return SUNcWilsonLines::VLeft->V;
    case 17: *n_doubles = 2 * 9 * S; return SUNcWilsonLines::VRight->V;
    default: *n_doubles = 0; return nullptr;
  }
}

std::vector<std::vector<double>> ReadTable(const std::string& path) {
  std::vector<std::vector<double>> rows;
  std::ifstream in(path.c_str());
  std::string line;
  while (std::getline(in, line)) {
    std::istringstream ss(line);
    std::vector<double> row;
    double v;
    while (ss >> v) row.push_back(v);
    if (!row.empty()) rows.push_back(row);
  }
  return rows;
}
}  // namespace

extern "C" {

void ref_set_outdir(const char* dir) {
  g_outdir = dir;
  IO::OutputDirectory = g_outdir + "/";
}

// Allocates the reference's global fields (S/Simulation.cpp:115-130 plus FourierSpace::Init).
void ref_init(const int* N, const double* a) {
  for (int i = 0; i < 3; i++) {
    Lattice::N[i] = N[i];
    Lattice::a[i] = a[i];
  }
  Lattice::Init();
  GaugeTransformation::Init();
  GaugeFixedVariables::Init();
  FourierSpace::Init();
  IO::OutputDirectory = g_outdir + "/";
  g_ready = true;
}

long ref_field_size(int which) {
  long n = 0;
  FieldPointer(which, &n);
  return n;
}
void ref_set_field(int which, const double* data) {
  long n = 0;
  void* p = FieldPointer(which, &n);
  std::memcpy(p, data, n * sizeof(double));
}
void ref_get_field(int which, double* data) {
  long n = 0;
  void* p = FieldPointer(which, &n);
  std::memcpy(data, p, n * sizeof(double));
}

void ref_set_threads(int n) { omp_set_num_threads(n); }

// IO::SaveConfiguration and IO::SaveConfigurationJ (S/IO/SaveConfiguration.cpp:6-93): the files are
// <outdir>/<stem>ID<seed>.txt.
void ref_save_configuration(const char* u_stem, const char* e_stem, const char* j_stem) {
  IO::SaveConfiguration(u_stem, e_stem);
  IO::SaveConfigurationJ(j_stem);
}
// IO::LoadConfiguration (S/IO/LoadConfiguration.cpp:190-200) from full paths; exits on malformed files.
void ref_load_configuration(const char* u_path, const char* e_path, const char* j_path) {
  IO::LoadConfiguration(u_path, e_path, j_path);
}

// nsteps x Dynamics::SUNc::Update (S/DYNAMICS/SUNcDynamics.cpp:353-378); returns seconds spent.
double ref_update(int nsteps, double dt) {
  Dynamics::dTStep = dt;
  const double t0 = omp_get_wtime();
  for (int n = 0; n < nsteps; n++)
    Dynamics::SUNc::Update(SUNcGaugeLinks::U, SUNcElectricFields::E, SUNcChargeDensity::Jp, SUNcChargeDensity::Jm,
                           SUNcChargeDensity::JpStat, SUNcChargeDensity::JmStat);
  return omp_get_wtime() - t0;
}

void ref_bulk(double* out) {
  Observables::Bulk::Update();
  for (int i = 0; i < 3; i++) {
    out[i] = Observables::Bulk::ESqr[i];
    out[3 + i] = Observables::Bulk::BSqr[i];
    out[6 + i] = Observables::Bulk::EDotJ[i];
  }
  out[9] = Observables::Bulk::T00();
  out[10] = Observables::Bulk::TXX();
  out[11] = Observables::Bulk::TYY();
  out[12] = Observables::Bulk::TZZ();
  out[13] = Observables::Bulk::ELECTRIC();
  out[14] = Observables::Bulk::MAGNETIC();
  out[15] = Observables::Bulk::SOURCE();
}

// Global Gauss-law violation (S/OBSERVABLES/GaussLawViolation.cpp:75-124).
void ref_gauss(double* mx, double* avg) {
  Observables::GaussLaw::UpdateViolation(0, Lattice::N[0] - 1, 0, Lattice::N[1] - 1, 0, Lattice::N[2] - 1,
                                         SUNcGaugeLinks::U, SUNcElectricFields::E, SUNcChargeDensity::JpStat,
                                         SUNcChargeDensity::JmStat);
  *mx = Observables::GaussLaw::GlobalMaxViolation;
  *avg = Observables::GaussLaw::GlobalAvgViolation;
}

// Per-z Gauss-law profile (:16-72); the reference writes it to a text file at 15 digits.
void ref_gauss_profile(double* zprof) {
  Observables::GaussLaw::UpdateViolation(0, Lattice::N[0] - 1, 0, Lattice::N[1] - 1, 0, Lattice::N[2] - 1,
                                         SUNcGaugeLinks::U, SUNcElectricFields::E, SUNcChargeDensity::JpStat,
                                         SUNcChargeDensity::JmStat, std::string("HarnessGaussProfile"));
  auto rows = ReadTable(IO::OutputDirectory + "HarnessGaussProfileID" + std::to_string(RandomNumberGenerator::MySEED) + ".txt");
  for (size_t i = 0; i < rows.size(); i++) zprof[(int)rows[i][0]] = rows[i][1];
}

void ref_unitarity(double* mx, double* avg) {
  Observables::Unitarity::UpdateViolation(0, Lattice::N[0] - 1, 0, Lattice::N[1] - 1, 0, Lattice::N[2] - 1,
                                          SUNcGaugeLinks::U);
  *mx = Observables::Unitarity::GlobalMaxViolation;
  *avg = Observables::Unitarity::GlobalAvgViolation;
}

// EnergyMomentumTensor::CreateMap (S/OBSERVABLES/EnergyMomentumTensor.cpp:92-170), read back from its file.
void ref_emt_map(double* out) {
  Observables::EnergyMomentumTensor::CreateMap(std::string("HarnessEMT"));
  auto rows = ReadTable(IO::OutputDirectory + "HarnessEMTID" + std::to_string(RandomNumberGenerator::MySEED) + ".txt");
  for (size_t i = 0; i < rows.size(); i++)
    for (int k = 0; k < 10; k++) out[10 * (int)rows[i][0] + k] = rows[i][1 + k];
}

// CoulombGaugeFixing::SetCoulombGauge (S/GAUGETRANSFORMATION/CoulombGaugeFixing.cpp:32-88) with the
// step size alphaStepSize; log rows (n, maxdev, avgdev, maxstep, avgstep, minF, sumF/V) read back.
int ref_coulomb(double alpha, int total_steps, double* log_out, int max_rows) {
  CoulombGaugeFixing::FourierAccelerationAlgorithm::alphaStepSize = alpha;
  CoulombGaugeFixing::SetCoulombGauge(std::string("HarnessCoulomb"), total_steps);
  auto rows = ReadTable(IO::OutputDirectory + "HarnessCoulombID" + std::to_string(RandomNumberGenerator::MySEED) + ".log");
  int n = 0;
  for (size_t i = 0; i < rows.size() && n < max_rows; i++, n++)
    for (int k = 0; k < 7 && k < (int)rows[i].size(); k++) log_out[7 * n + k] = rows[i][k];
  return n;
}

// Per-slice Coulomb gauge deviation of the reference's gauge-fixed links GaugeFixedVariables::U, with
// its own deviation macro GET_LOCAL_GAUGE_VIOLATION (S/GAUGETRANSFORMATION/CoulombGaugeDeviation.cpp:23-41):
// zmax[z] = max |Delta^a|, zsq[z] = sum Delta^a^2 over slice z.
void ref_coulomb_profile(double* zmax, double* zsq) {
  using namespace CoulombGaugeFixing;
  GaugeLinks* UGaugeTransformed = GaugeFixedVariables::U;
  SET_GAUGE_DEVIATION_BUFFERS();
  for (int z = 0; z < Lattice::N[2]; z++) {
    double mx = 0.0, sq = 0.0;
    for (int y = 0; y < Lattice::N[1]; y++)
      for (int x = 0; x < Lattice::N[0]; x++) {
        GET_LOCAL_GAUGE_VIOLATION(x, y, z);
        for (int a = 0; a < SUNcAlgebra::NumberOfGenerators; a++) {
          mx = std::max(mx, std::abs(DeviationBuffer[a]));
          sq += DeviationBuffer[a] * DeviationBuffer[a];
        }
      }
    zmax[z] = mx;
    zsq[z] = sq;
  }
}

// SetCoulombGauge's loop (S/GAUGETRANSFORMATION/CoulombGaugeFixing.cpp:32-88) around one of the
// reference's own updates: the Fourier-accelerated one (algorithm 0, param = alphaStepSize), Los Alamos
// (1, param = OverRelaxationProbability) or Jacobi (2, param = alphaStepSize).  The reference selects its
// algorithm with a #define inside CoulombGaugeFixing.cpp and logs with the stream's default 6 digits, so
// the loop is restated here; the log rows come from the Global* monitors at full precision, into log_out
// and, row by row and flushed, into <outdir>/HarnessCoulombRows.txt (which survives the exit(0) of the
// unitarity guard).  uniforms: the values rng() returns, in call order.
int ref_coulomb_local(int algorithm, double param, const double* uniforms, long n_uniforms, int total_steps,
                      double* log_out, int max_rows) {
  RandomNumberGenerator::Uniforms.assign(uniforms, uniforms + n_uniforms);
  RandomNumberGenerator::UniformCursor = 0;
  if (algorithm == 0)
    CoulombGaugeFixing::FourierAccelerationAlgorithm::alphaStepSize = param;
  else if (algorithm == 1)
    CoulombGaugeFixing::LosAlamosAlgorithm::OverRelaxationProbability = param;
  else
    CoulombGaugeFixing::JacobiAlgorithm::alphaStepSize = param;
  FILE* rows = std::fopen((g_outdir + "/HarnessCoulombRows.txt").c_str(), "w");
  GaugeTransformation::Operations::CopyFields();
  GaugeTransformation::Operations::GaugeTransformLinks();
  CoulombGaugeFixing::GlobalMaxDeviation = 1;
  int n = 0;
  while (n < total_steps && CoulombGaugeFixing::GlobalMaxDeviation > std::pow(10.0, -15)) {
    if (algorithm == 0)
      CoulombGaugeFixing::FourierAccelerationAlgorithm::UpdateGaugeTransformation();
    else if (algorithm == 1)
      CoulombGaugeFixing::LosAlamosAlgorithm::UpdateGaugeTransformation();
    else
      CoulombGaugeFixing::JacobiAlgorithm::UpdateGaugeTransformation();
    const double row[7] = {(double)n,
                           CoulombGaugeFixing::GlobalMaxDeviation,
                           CoulombGaugeFixing::GlobalAvgDeviation,
                           CoulombGaugeFixing::GlobalMaxStepSize,
                           CoulombGaugeFixing::GlobalAvgStepSize,
                           CoulombGaugeFixing::GlobalMinGaugeFunctional,
                           CoulombGaugeFixing::GlobalSumGaugeFunctional};
    if (n < max_rows)
      for (int k = 0; k < 7; k++) log_out[7 * n + k] = row[k];
    if (rows) {
      for (int k = 0; k < 7; k++) std::fprintf(rows, k ? " %.17g" : "%.17g", row[k]);
      std::fprintf(rows, "\n");
      std::fflush(rows);
    }
    n++;
  }
  if (rows) std::fclose(rows);
  GaugeTransformation::Operations::GaugeTransformLinks();
  GaugeTransformation::Operations::GaugeTransformElectricFields();
  return n;
}

void ref_expi(double c, const double* alpha, double* out18) {
  SUNcAlgebra::Operations::MatrixIExp(c, const_cast<double*>(alpha), reinterpret_cast<COMPLEX*>(out18));
}
void ref_matrix_ilog(double c, const double* W18, double* out8) {
  SUNcAlgebra::Operations::MatrixILog(c, reinterpret_cast<COMPLEX*>(const_cast<double*>(W18)), out8);
}

// MV collision initial state as in Simulation::Run (S/Simulation.cpp:337-374): SetWilsonLines for the
// left and the right nucleus (consuming 8*Nx*Ny injected Gaussians each, in the reference's loop order
// y, x, a), then SingleSheet for z in [0,(Nz-2)/2] ('L') and [Nz/2,Nz-1] ('R'), then ghost syncs.
// single_left != 0 gives the one-nucleus set-up of S/LeftNucleusSimulation.cpp instead (SingleSheet 'L'
// over all z, no right nucleus).
void ref_mv_init(const double* gauss, long n_gauss, double dt, double qsL, double qsR, int centerL, int centerR,
                 double sigma, double lambda, double meff, int single_left) {
  RandomNumberGenerator::Injected.assign(gauss, gauss + n_gauss);
  RandomNumberGenerator::Cursor = 0;
  Dynamics::dTStep = dt;
  Dynamics::Reset();
  Parameters::SigmaLOverAzL = sigma;
  Parameters::SigmaLOverAzR = sigma;
  Parameters::Lambda = lambda;
  Parameters::MEff = meff;
  CollidingObjects::SetWilsonLines(SUNcChargeDensity::rhoOldL, SUNcChargeDensity::rhoL, SUNcWilsonLines::VLeft, 'L',
                                   centerL, qsL);
  if (single_left) {
    InitialConditions::SingleSheet::SingleSheet(SUNcChargeDensity::rhoL, 0, Lattice::N[2] - 1, SUNcChargeDensity::RhoLT1,
                                                SUNcWilsonLines::VLeft, 'L', SUNcChargeDensity::JpStat, SUNcChargeDensity::Jp);
  } else {
    CollidingObjects::SetWilsonLines(SUNcChargeDensity::rhoOldR, SUNcChargeDensity::rhoR, SUNcWilsonLines::VRight, 'R',
                                     centerR, qsR);
    InitialConditions::SingleSheet::SingleSheet(SUNcChargeDensity::rhoL, 0, (Lattice::N[2] - 2) / 2,
                                                SUNcChargeDensity::RhoLT1, SUNcWilsonLines::VLeft, 'L',
                                                SUNcChargeDensity::JpStat, SUNcChargeDensity::Jp);
    InitialConditions::SingleSheet::SingleSheet(SUNcChargeDensity::rhoR, Lattice::N[2] / 2, Lattice::N[2] - 1,
                                                SUNcChargeDensity::RhoRT1, SUNcWilsonLines::VRight, 'R',
                                                SUNcChargeDensity::JmStat, SUNcChargeDensity::Jm);
  }
  SUNcChargeDensity::JpStat->SynchronizeGhostCells();
  SUNcChargeDensity::Jp->SynchronizeGhostCells();
  SUNcChargeDensity::JmStat->SynchronizeGhostCells();
  SUNcChargeDensity::Jm->SynchronizeGhostCells();
  SUNcGaugeLinks::U->SynchronizeGhostCells();
  SUNcGaugeLinks::UOld->SynchronizeGhostCells();
  SUNcElectricFields::E->SynchronizeGhostCells();
}

// The TMD / Glauber initial state of SimulationmitPC::Run (S/SimulationmitPC.cpp:315-367): per nucleus
// ChargeDistributions::ChargeFluctuation (S/TMDNUCLEUS/CorrelationFunction.cpp:23-97) and
// TmdBasedCollision::SetWilsonLines (S/TMDNUCLEUS/TMDbased.cpp:243-291, its Nucleus sampled as in
// S/TMDNUCLEUS/GBWSampling.cpp), left first; then SingleSheet for both nuclei and the ghost syncs.
// gauss: the Gauss() values in call order (8 Nx Ny Nz per nucleus); uniforms: the rng() values (the
// nucleon positions).  The Parameters the reference derives at static initialisation are set here.
void ref_tmd_init(const double* gauss, long n_gauss, const double* uniforms, long n_uniforms, double dt, int A,
                  double qs0a, double meff, double ax_fm, double ay_fm, double az_fm, double com_energy) {
  RandomNumberGenerator::Injected.assign(gauss, gauss + n_gauss);
  RandomNumberGenerator::Cursor = 0;
  RandomNumberGenerator::Uniforms.assign(uniforms, uniforms + n_uniforms);
  RandomNumberGenerator::UniformCursor = 0;
  Dynamics::dTStep = dt;
  Dynamics::Reset();
  Parameters::AtomicNumber = A;
  Parameters::Qs0A = qs0a;
  Parameters::MEff = meff;
  Parameters::aXInFm = ax_fm;
  Parameters::aYInFm = ay_fm;
  Parameters::aZInFm = az_fm;
  Parameters::CoMEnergy = com_energy;
  ChargeDistributions::ChargeFluctuation(SUNcChargeDensity::CFL, 'L');
  SUNcChargeDensity::CFL->SynchronizeGhostCells();
  TmdBasedCollision::SetWilsonLines(SUNcChargeDensity::rhoL, SUNcChargeDensity::CFL, SUNcWilsonLines::VLeft, 'L');
  SUNcChargeDensity::rhoL->SynchronizeGhostCells();
  ChargeDistributions::ChargeFluctuation(SUNcChargeDensity::CFR, 'R');
  SUNcChargeDensity::CFR->SynchronizeGhostCells();
  TmdBasedCollision::SetWilsonLines(SUNcChargeDensity::rhoR, SUNcChargeDensity::CFR, SUNcWilsonLines::VRight, 'R');
  SUNcChargeDensity::rhoR->SynchronizeGhostCells();
  InitialConditions::SingleSheet::SingleSheet(SUNcChargeDensity::rhoL, 0, (Lattice::N[2] - 2) / 2,
                                              SUNcChargeDensity::RhoLT1, SUNcWilsonLines::VLeft, 'L',
                                              SUNcChargeDensity::JpStat, SUNcChargeDensity::Jp);
  InitialConditions::SingleSheet::SingleSheet(SUNcChargeDensity::rhoR, Lattice::N[2] / 2, Lattice::N[2] - 1,
                                              SUNcChargeDensity::RhoRT1, SUNcWilsonLines::VRight, 'R',
                                              SUNcChargeDensity::JmStat, SUNcChargeDensity::Jm);
  SUNcChargeDensity::JpStat->SynchronizeGhostCells();
  SUNcChargeDensity::Jp->SynchronizeGhostCells();
  SUNcChargeDensity::JmStat->SynchronizeGhostCells();
  SUNcChargeDensity::Jm->SynchronizeGhostCells();
  SUNcGaugeLinks::U->SynchronizeGhostCells();
  SUNcGaugeLinks::UOld->SynchronizeGhostCells();
  SUNcElectricFields::E->SynchronizeGhostCells();
}

// How many rng() values the last run consumed (the rejection sampling's count is not known in advance).
long ref_uniforms_used() { return (long)RandomNumberGenerator::UniformCursor; }

}  // extern "C"
