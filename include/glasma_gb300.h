/* glasma_gb300.h -- C ABI of the GB300 real-time SU(3) glasma library.
 *
 * One handle = one lattice resident in GPU memory.  Every entry point returns an
 * int status (GLASMA_OK = 0) and never exits the process; glasma_last_error()
 * gives a message for the last failure on the calling thread.
 *
 * The reference program has no library boundary: its hot path is a set of C++
 * namespaces compiled as one translation unit and driven by Simulation::Evolve
 * (S/Simulation.cpp:212-321; S/ = the reference's SourceCode directory).  Each
 * entry point below names the reference function it stands in for.  The C++
 * drop-in shim with the reference's own class and namespace names is
 * glasma_gb300_reference_api.hpp.
 *
 * Host buffers passed to upload/download use the reference's host layout, FP64,
 * ghost slices included (S = Nx*Ny*(Nz+2) sites, site s = x + Nx*(y + Ny*(z+1))):
 *   GLASMA_FIELD_U, _UOLD, _UG   complex double [S][3][9], element (i,j) at i+3j
 *                                 (S/LATTICE/GaugeLinks.cpp:38-41)
 *   GLASMA_FIELD_E, _EG           double [S][3][8]  (S/LATTICE/ElectricFields.cpp:31-35)
 *   GLASMA_FIELD_JP ... _JMSTAT   double [S][8]     (S/LATTICE/ChargeDensity.cpp:24-33)
 *   GLASMA_FIELD_G                complex double [S][9] (S/LATTICE/GaugeTransformations.cpp:25-38)
 * Calls on one handle are not re-entrant; each handle issues its work on one CUDA
 * stream (its own, or the one given to glasma_set_stream).
 */
#ifndef GLASMA_GB300_H
#define GLASMA_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct glasma_lattice glasma_lattice;

enum glasma_status {
  GLASMA_OK = 0,
  GLASMA_ERR_INVALID_ARGUMENT = 1, /* null handle / pointer, unknown field or flag    */
  GLASMA_ERR_BAD_SHAPE = 2,        /* lattice extent or spacing out of range          */
  GLASMA_ERR_OUT_OF_MEMORY = 3,    /* device allocation failed                        */
  GLASMA_ERR_CUDA = 4,             /* a CUDA call or kernel launch failed             */
  GLASMA_ERR_NUMERICAL = 5,        /* numerical guard fired (reference: exit(0))      */
  GLASMA_ERR_TIMEOUT = 6,          /* a bounded device wait ran out                   */
  GLASMA_ERR_UNSUPPORTED = 7       /* operation not available for this handle         */
};

enum glasma_precision { GLASMA_FP64 = 0, GLASMA_FP32 = 1 };

enum glasma_field {
  GLASMA_FIELD_U = 0,
  GLASMA_FIELD_UOLD = 1,
  GLASMA_FIELD_E = 2,
  GLASMA_FIELD_JP = 3,
  GLASMA_FIELD_JM = 4,
  GLASMA_FIELD_JPSTAT = 5,
  GLASMA_FIELD_JMSTAT = 6,
  GLASMA_FIELD_G = 7,
  GLASMA_FIELD_UG = 8,
  GLASMA_FIELD_EG = 9
};

/* glasma_step flags */
#define GLASMA_STEP_SAVE_UOLD 0x1u /* write UOld = U(t+dt/2) of the last step (SaveOldLink) */

/* glasma_coulomb_fix_algorithm algorithms: the three updates of S/GAUGETRANSFORMATION/ALGORITHMS/
   (the reference compiles one, selected by a #define in CoulombGaugeFixing.cpp:4) */
#define GLASMA_GF_FOURIER 0    /* FourierAccelerationAlgorithm; param = alphaStepSize (reference 2.0) */
#define GLASMA_GF_LOS_ALAMOS 1 /* LosAlamosAlgorithm; param = OverRelaxationProbability (reference 0.0) */
#define GLASMA_GF_JACOBI 2     /* JacobiAlgorithm; param = alphaStepSize (reference 0.3) */

/* glasma_coulomb_fix flags */
#define GLASMA_GF_PROJECT_ZERO_MODE 0x1u /* drop the p=0 mode of the update (the reference keeps
                                            it unnormalised); a documented deviation */
#define GLASMA_GF_FFT_FP32 0x2u          /* run the acceleration step's two 3D transforms in FP32
                                            (the gradient, the update and the links stay FP64): the
                                            iterates differ from the reference's at the 1e-7 level,
                                            the converged gauge is the same */
#define GLASMA_GF_OPEN_Z 0x4u            /* open-z functional, a documented variant: the top slice's
                                            forward z link (into the ghost slice) is left out of the
                                            deviation (the reference counts it at one end only,
                                            CoulombGaugeDeviation.cpp:37, so its iteration does not
                                            converge with open z boundaries); Delta is then the
                                            gradient of sum Re tr UG over the links inside the lattice
                                            and the iteration converges */
#define GLASMA_GF_MIXED 0x8u             /* FP64 handles: the sweeps first run on FP32 copies of U and
                                            G in FP32 arithmetic (FP32 transforms, FP64 monitor sums)
                                            until the maximum deviation is <= 1e-5 or stops falling, then
                                            G is widened, projected onto SU(3) in FP64, and the FP64
                                            sweeps finish to the stopping rule; log rows and the count
                                            cover both phases.  The FP32 update's unitarity guard is
                                            1e-5.  GLASMA_ERR_UNSUPPORTED on FP32 handles */

/* Create a lattice (replaces Lattice::Init, S/LATTICE/SUNcVariables.cpp:71-90, and the
 * container constructors, S/LATTICE/GaugeLinks.cpp:110-127): links set to the identity,
 * E and the four currents to zero, ghost slices included.  precision: glasma_precision.
 * reunitarize_every: FP32 only, project the links back onto SU(3) after every n-th step
 * (0 = never).  Uses the current CUDA device. */
int glasma_create(int nx, int ny, int nz, double ax, double ay, double az, int precision, int reunitarize_every,
                  glasma_lattice** out);
int glasma_destroy(glasma_lattice* h);

/* Work is issued on `cuda_stream` (a cudaStream_t; NULL = the handle's own stream). */
int glasma_set_stream(glasma_lattice* h, void* cuda_stream);
/* The reference's Lattice::aScale (S/LATTICE/3DGrid.cpp:35-36), used by the observables. */
int glasma_set_scale(glasma_lattice* h, double a_scale);
int glasma_get_shape(const glasma_lattice* h, int* nx, int* ny, int* nz, int* precision);
/* Number of doubles of one field in the host layout (with ghost slices). */
long long glasma_field_doubles(const glasma_lattice* h, int field);

/* Copy a whole field, ghost slices included, from / to host memory in the reference's host
 * layout (replaces direct access to GaugeLinks::U, ElectricFields::E, ChargeDensity::J).
 * Pinned host memory makes the copy asynchronous up to the stream synchronisation that
 * download performs before it returns. */
int glasma_upload(glasma_lattice* h, int field, const double* host);
int glasma_download(glasma_lattice* h, int field, double* host);
/* Same, from / to a device buffer holding the host layout. */
int glasma_upload_device(glasma_lattice* h, int field, const double* device_aos);
/* Uploads that overlap the handle's kernels: glasma_upload_begin starts copying `host` (reference
 * layout, as for glasma_upload) into a staging area on the handle's own transfer stream and returns;
 * glasma_upload_finish orders the handle's stream after every begun copy and converts them into the
 * fields (on that stream, without waiting on the host).  Kernels enqueued before finish still see the
 * old fields, so the next step's inputs can travel while the current step runs:
 *   begin(inputs 0); finish(); for k: { begin(inputs k+1); step(); read result; finish(); }
 * The host buffers must stay unchanged until the handle's stream has passed finish's conversion (after
 * any synchronising call: an observable, a download, glasma_synchronize); page-locked buffers let the
 * copy run without the CPU.  The staging is double buffered (two sets of the begun fields' size, allocated
 * on first use): a begin waits on the device only for the conversion two finishes back, which has
 * normally long completed, so the copies start at once.
 * No reference counterpart (the reference's fields live on the host). */
int glasma_upload_begin(glasma_lattice* h, int field, const double* host);
int glasma_upload_finish(glasma_lattice* h);
int glasma_download_device(glasma_lattice* h, int field, double* device_aos);

/* nsteps x Dynamics::SUNc::Update (S/DYNAMICS/SUNcDynamics.cpp:353-378) with time step dt.
 * With the plaquette method (the default) a force kernel over the plaquettes and a link/J kernel
 * that gathers their contributions into E run per step (equal to the staple form up to rounding);
 * with the two-pass method the electric-field/JStat sub-steps and the link/J sub-steps are two
 * kernels working in place; with the one-pass method each step is one kernel that reads the links
 * and currents of time t from one set of buffers and writes those of t+dt to a second set, which
 * the handle allocates on first use and swaps with the first after every step.  Two-pass and
 * one-pass give bit-identical fields.  SaveOldLink runs when GLASMA_STEP_SAVE_UOLD is set (for
 * the last step of the call, which leaves UOld exactly as the reference leaves it). */
int glasma_step(glasma_lattice* h, double dt, int nsteps, unsigned flags);

/* Step method of the handle: GLASMA_STEP_PLAQUETTE (default), GLASMA_STEP_TWO_PASS (no extra memory) or
 * GLASMA_STEP_ONE_PASS (half the HBM traffic per step, 2 x (U + 4 currents) per site more memory;
 * falls back to two-pass for a call when the second buffer set cannot be allocated), or
 * GLASMA_STEP_PLAQUETTE: the electric force summed plaquette by plaquette (each site's three
 * plaquettes and six adjoint rotations instead of twelve staples; the same terms regrouped, equal to
 * the other methods up to rounding), two kernels per step, 48 reals per site more memory (falls back
 * to two-pass for a call when that cannot be allocated).  GLASMA_STEP_MARCH: the plaquette method in
 * one kernel per step, each block marching along z through a tile of (x, y) sites (the rotated force
 * terms handed over in shared memory and registers instead of HBM); equal to GLASMA_STEP_PLAQUETTE
 * up to rounding, with the one-pass method's second buffer set (falls back to two-pass for a
 * call when that cannot be allocated).
 * glasma_get_step_method reports the method the last glasma_step call used. */
#define GLASMA_STEP_ONE_PASS 0
#define GLASMA_STEP_TWO_PASS 1
#define GLASMA_STEP_PLAQUETTE 2
#define GLASMA_STEP_MARCH 3
int glasma_set_step_method(glasma_lattice* h, int method);
int glasma_get_step_method(glasma_lattice* h, int* method);
/* z slices each block of GLASMA_STEP_MARCH walks (0, the default: chosen from the lattice so that the
 * blocks fill the GPU); a tuning knob, the fields do not depend on it.  No reference counterpart. */
int glasma_set_march_chunk(glasma_lattice* h, int slices);

/* Link storage of the leapfrog step (FP32 handles): 18 reals per link (default) or 12, rows 0 and 1
 * of each link, with row 2 formed in registers as the unitary complement conj(row0 x row1).  With 12
 * the step kernels and the in-step reunitarisation read and write two thirds of the link bytes; at the
 * end of every glasma_step call row 2 is written back, so every other call sees full links.  Rows 0
 * and 1 are taken as the link: a link that is not in SU(3) when the call starts is replaced by the
 * SU(3)-completion of its first two rows.  GLASMA_ERR_UNSUPPORTED for 12 on FP64 handles (their
 * kernels are bound by the FP64 pipe, which the reconstruction would load further).
 * No reference counterpart (the reference stores full links, S/LATTICE/GaugeLinks.cpp). */
int glasma_set_link_storage(glasma_lattice* h, int reals_per_link);

/* Arithmetic of the plaquette method's force kernel on FP64 handles: GLASMA_FP64_NATIVE (default) or
 * GLASMA_FP64_DOUBLE_FLOAT, double-float arithmetic on the FP32 pipe (each value an unevaluated sum of
 * two floats, ~48-bit significand; the FP64 fields are converted on load and store).  GB300 runs FP64
 * at 1/64 of its FP32 rate.  Ignored by FP32 handles and the other step methods. */
#define GLASMA_FP64_NATIVE 0
#define GLASMA_FP64_DOUBLE_FLOAT 1
int glasma_set_fp64_arithmetic(glasma_lattice* h, int mode);
int glasma_get_fp64_arithmetic(glasma_lattice* h, int* mode);
int glasma_get_link_storage(glasma_lattice* h, int* reals_per_link);

/* glasma_step with CUDA events recorded on the handle's stream around the kernels of every
 * step; kernel_ms[0] / kernel_ms[1] receive the summed milliseconds of the electric-field/JStat
 * kernel and of the link/J kernel (two-pass; for the plaquette method its force kernel and its
 * gathering link/J kernel), or of the one-pass kernel and 0 (one-pass).
 * Waits for the last event. */
int glasma_step_profiled(glasma_lattice* h, double dt, int nsteps, unsigned flags, double* kernel_ms);

/* The individual sub-steps, each with the reference's ghost synchronisation:
 * UpdateElectricFields (:134-203), UpdateJStat (:205-236), UpdateGaugeLinks(dt_arg) (:62-106;
 * U <- exp(i (-dt_arg a_mu^2/a^3) t.E_mu) U), SaveOldLink (:108-128), UpdateJ (:238-269). */
int glasma_update_efield(glasma_lattice* h, double dt);
int glasma_update_jstat(glasma_lattice* h, double dt);
int glasma_update_links(glasma_lattice* h, double dt_arg);
int glasma_save_old_link(glasma_lattice* h);
int glasma_update_j(glasma_lattice* h, double dt);

/* Observables::Bulk::Update and its accessors (S/OBSERVABLES/BulkObservables.cpp:22-183).
 * out[0..2] ESqr, [3..5] BSqr, [6..8] EDotJ, [9..15] T00, TXX, TYY, TZZ, ELECTRIC, MAGNETIC, SOURCE
 * (volume sums, as the reference returns them). */
int glasma_bulk(glasma_lattice* h, double out[16]);
/* Observables::GaussLaw::UpdateViolation (S/OBSERVABLES/GaussLawViolation.cpp:16-124).
 * sync_first != 0 first syncs the ghosts of JpStat, JmStat, U and E (as the per-z form does).
 * zprofile (may be NULL): Nz doubles, sum_{x,y,a} G^2 / (Nx Ny) per slice. */
int glasma_gauss(glasma_lattice* h, int sync_first, double* max_violation, double* avg_violation, double* zprofile);
/* Observables::Unitarity::UpdateViolation (S/OBSERVABLES/UnitarityViolation.cpp:13-51). */
int glasma_unitarity(glasma_lattice* h, double* max_violation, double* avg_violation);
/* Observables::EnergyMomentumTensor::CreateMap (S/OBSERVABLES/EnergyMomentumTensor.cpp:92-170):
 * out[z*10 + k], k = T00, TXX, TYY, TZZ, T0X, T0Y, T0Z, TXY, TYZ, TZX (transverse averages). */
int glasma_emt_map(glasma_lattice* h, double* out);
/* Pressure anisotropy of the slices z in [z_begin, z_end): P_L = mean TZZ, P_T = mean (TXX+TYY)/2
 * from the CreateMap columns (S/OBSERVABLES/EnergyMomentumTensor.cpp:140-142), ratio = P_L / P_T.
 * No reference function computes it; it is the late-time objective of the adjoint configuration. */
int glasma_pressure_anisotropy(glasma_lattice* h, int z_begin, int z_end, double* ratio, double* p_l, double* p_t);

/* Project every link onto SU(3) (Gram-Schmidt on two rows, third row from their cross product). */
int glasma_reunitarize(glasma_lattice* h);

/* CoulombGaugeFixing::SetCoulombGauge (S/GAUGETRANSFORMATION/CoulombGaugeFixing.cpp:32-88) with
 * the Fourier-accelerated update (S/GAUGETRANSFORMATION/ALGORITHMS/FourierAcceleration.cpp:15-142).
 * alpha: the reference's alphaStepSize.  Iterates while n < max_iters and the latest maximum
 * deviation > tol (the reference uses 1e-15).  The gauge transformation G persists in the handle
 * across calls (identity at creation, reset with glasma_gauge_reset); the gauge-fixed links and
 * fields are GLASMA_FIELD_UG / GLASMA_FIELD_EG.  log (may be NULL): max_iters x 7 doubles per
 * iteration: n, max dev, avg dev, max step, avg step, min functional, sum functional / V.
 * Returns GLASMA_ERR_NUMERICAL when an update leaves unitarity by more than 1e-13 (the reference
 * exits there). */
int glasma_coulomb_fix(glasma_lattice* h, double alpha, int max_iters, double tol, unsigned flags, double* log,
                       int* iterations);
/* SetCoulombGauge with any of the reference's three updates (S/GAUGETRANSFORMATION/ALGORITHMS/):
 *   GLASMA_GF_FOURIER     glasma_coulomb_fix(h, param, max_iters, tol, flags, ...)
 *   GLASMA_GF_LOS_ALAMOS  LosAlamosAlgorithm::UpdateGaugeTransformation (LosAlamos.cpp:13-95): the even
 *                         sites ((x+y+z) even), links re-transformed, the odd sites, links re-transformed;
 *                         per site G <- P(w)^d G with P = SUNcGroup::Extended::MaxTraceProjection
 *                         (S/SUNc/SU3/GroupOperations.cpp:358-378, seven Cabibbo-Marinari sweeps), or
 *                         G <- P^d P^d G (over-relaxation) when the site's draw is <= param.  The draws
 *                         are a counter-based hash of (seed, 2*iteration + pass, site): reproducible, and
 *                         independent of the order the sites are visited in (the reference's rng() stream
 *                         depends on its OpenMP schedule).  With param = 0 (the reference's value) no draw
 *                         matters and the iterates are the reference's.
 *   GLASMA_GF_JACOBI      JacobiAlgorithm::UpdateGaugeTransformation (Jacobi.cpp:13-80): every site at once,
 *                         G <- exp(-i param t.Delta)^d G.
 * flags: Fourier only (0 otherwise).  Log rows, stopping rule, G persistence and the unitarity guard as
 * for glasma_coulomb_fix. */
int glasma_coulomb_fix_algorithm(glasma_lattice* h, int algorithm, double param, unsigned long long seed, int max_iters,
                                 double tol, unsigned flags, double* log, int* iterations);
/* GaugeTransformation::SetIdentity (S/GAUGETRANSFORMATION/GaugeTransformation.cpp:41-60). */
int glasma_gauge_reset(glasma_lattice* h);
/* The handle's gauge transformation G applied to one colour-charge field, PERFORM_COLOR_CHARGE_TRANSFORMATION
 * (S/CALC/GaugeTransformation.cpp:28-31; the colour-current form :20-25 is the same action per component):
 * jG(x) = AdjointMultiplication(G(x), j(x)) = 2 tr(t^a G (t.j) G^dagger) for field GLASMA_FIELD_JP ..
 * GLASMA_FIELD_JMSTAT, written to out (host or device memory, S x 8 doubles in the field's host layout;
 * the ghost slices take the edge slices' values).  The handle's fields are not changed. */
int glasma_transform_charge(glasma_lattice* h, int field, double* out);

/* McLerran-Venugopalan initial state, as Simulation::Run builds it (S/Simulation.cpp:337-374:
 * CollidingObjects::SetWilsonLines for each nucleus, then SingleSheet over z in [0,(Nz-2)/2] for
 * the left and [Nz/2,Nz-1] for the right nucleus) or, with single_left != 0, one left-moving nucleus
 * over all z (S/LeftNucleusSimulation.cpp).  zeta_left / zeta_right: the charge fluctuations the
 * reference draws from its random generator (S/COLLIDINGOBJECTS/CollidingObjects.cpp:335-342), host
 * arrays of 8*Nx*Ny N(0,1) numbers in its order a + 8*(x + Nx*y); qs scales them (g^2 mu), centre and
 * sigma give the longitudinal profile, lambda and meff the smoothing, dt the time step of the
 * evolved sheet.  Overwrites U, UOld, E and the four currents; ghost slices synced. */
int glasma_mv_init(glasma_lattice* h, int single_left, const double* zeta_left, const double* zeta_right,
                   double qs_left, double qs_right, int center_left, int center_right, double sigma, double lambda,
                   double meff, double dt);
const char* glasma_mv_last_error(void);

/* Parameters of the TMD / Glauber initial state, under the reference's names (S/LATTICE/Parameters.cpp
 * and the nuclear centres of S/TMDNUCLEUS/TMDbased.cpp:41-50); the reference's values in brackets for
 * a = 1.  glasma_tmd_default_params fills them. */
typedef struct {
  int atomic_number;   /* Parameters::AtomicNumber [197]; 16, 54, 197 or 208 (NuclearData.cpp) */
  double qs0a;         /* Parameters::Qs0A, lattice units [0.33] */
  double meff;         /* Parameters::MEff, infrared cut-off of the 2D filter [Qs0A] */
  double ax_fm, ay_fm; /* Parameters::aXInFm, aYInFm [Qs0A 0.197 / 0.5] */
  double az_fm;        /* Parameters::aZInFm [aXInFm / (Qs0A 512)] */
  double com_energy;   /* Parameters::CoMEnergy in fm^-1 [500 / 0.197]; Lorentz factor = com_energy 0.197 / 2 */
  int center_left;     /* slice of the left nucleus' centre [785] */
  int center_right;    /* slice of the right nucleus' centre [1261] */
  double dt;           /* Dynamics::dTStep of the first step (SingleSheet) */
} glasma_tmd_params;

void glasma_tmd_default_params(glasma_tmd_params* p, double dt);

/* The Woods-Saxon nucleus of Nucleus::SetNucleonPositions (S/TMDNUCLEUS/GBWSampling.cpp:20-84):
 * rejection sampling of A nucleons from the uniform draws the reference takes from rng() (four per
 * trial: x, y, z in [-4R, 4R), acceptance), then the centre of mass moved to the origin.  positions:
 * A x 3 doubles in fm; used (may be NULL): draws consumed.  Host only.  GLASMA_ERR_INVALID_ARGUMENT
 * when A has no Woods-Saxon entry or the draws run out. */
int glasma_glauber_sample(int A, const double* uniforms, long n_uniforms, double* positions, long* used);

/* The TMD / Glauber initial state of SimulationmitPC::Run (S/SimulationmitPC.cpp:315-367): per nucleus
 * ChargeDistributions::ChargeFluctuation (S/TMDNUCLEUS/CorrelationFunction.cpp:23-97) from the injected
 * noise, TmdBasedCollision::SetWilsonLines (S/TMDNUCLEUS/TMDbased.cpp:243-291) with the given nucleons,
 * then InitialConditions::SingleSheet for both nuclei and the ghost syncs.  noise_left / noise_right:
 * 8 Nx Ny Nz N(0,1) numbers each, in the order the reference draws them (index a + 8 (x + Nx (y + Ny z)));
 * nucleons_left / nucleons_right: A x 3 positions (glasma_glauber_sample).  rho_left / rho_right (may be
 * NULL): receive the filtered densities SUNcChargeDensity::rhoL / rhoR (8 doubles per site, ghost slices
 * included).  Host arrays. */
int glasma_tmd_init(glasma_lattice* h, const double* noise_left, const double* noise_right,
                    const double* nucleons_left, const double* nucleons_right, const glasma_tmd_params* params,
                    double* rho_left, double* rho_right);

/* Configuration files in the reference's text format: IO::SaveConfiguration and
 * IO::SaveConfigurationJ (S/IO/SaveConfiguration.cpp:6-93) write the links, E and the four currents
 * one entry per line, ghost slices included, with 15 significant digits; IO::LoadConfiguration
 * (S/IO/LoadConfiguration.cpp:3-200) reads them back.  Any path may be NULL to skip that file.
 * Reading checks the entries' order and count and returns GLASMA_ERR_INVALID_ARGUMENT (message in
 * glasma_io_last_error) where the reference exits; it reads all eight colours of the currents file
 * (the reference's loader fills colours 0-2 only) and uploads nothing unless every file read cleanly.
 * The _host forms work on host arrays in the reference's layout and need no GPU. */
int glasma_save_text(glasma_lattice* h, const char* links_path, const char* efield_path, const char* currents_path);
int glasma_load_text(glasma_lattice* h, const char* links_path, const char* efield_path, const char* currents_path);
int glasma_write_text_host(int nx, int ny, int nz, const double* U, const double* E, const double* JpStat,
                           const double* Jp, const double* JmStat, const double* Jm, const char* links_path,
                           const char* efield_path, const char* currents_path);
int glasma_read_text_host(int nx, int ny, int nz, double* U, double* E, double* JpStat, double* Jp, double* JmStat,
                          double* Jm, const char* links_path, const char* efield_path, const char* currents_path);
/* Binary restart file (no reference counterpart): U, UOld, E and the four currents in the
 * reference's host layout after a 64-byte header (lattice shape, spacings, step count); loading
 * reproduces the fields bit for bit.  The lattice shape must match the handle's. */
int glasma_save_binary(glasma_lattice* h, const char* path);
int glasma_load_binary(glasma_lattice* h, const char* path);
const char* glasma_io_last_error(void);

/* Seeded synthetic fields generated on the device (benchmarks, demos): links exp(i link_amp t.r),
 * E = e_amp r, the four currents j_amp r, r ~ N(0,1) from a counter-based generator (SplitMix64 +
 * Box-Muller), ghost slices synced.  Same seed, same fields.  No reference counterpart. */
int glasma_fill_synthetic(glasma_lattice* h, unsigned long long seed, double link_amp, double e_amp, double j_amp);

/* Autotuner: times the step kernel of the handle's step method (the one-pass kernel, or the
 * electric-field kernel of the two-pass method), computing and storing nothing, for each block
 * tile shape tile_x x (128/tile_x) sites of a z slice and keeps the fastest for this lattice;
 * *tile_x (may be NULL) receives it.  The plaquette method's kernels are pointwise: for it the
 * current tile is kept and reported without timing.  glasma_set_tile sets it by hand (tile_x
 * divides 128). */
int glasma_autotune(glasma_lattice* h, double dt, int* tile_x);
int glasma_set_tile(glasma_lattice* h, int tile_x);

/* The batched 3D FFT used by the gauge fixer, exposed for testing: 8 colour planes of complex
 * doubles, X[a][z][y][x] (8*Nx*Ny*Nz complex values, interleaved re/im), unnormalised,
 * exponent sign -1 (inverse = 0) or +1 (inverse = 1), the convention of FFTW's
 * fftw_plan_many_dft as S/FFT/FFT3D.cpp:126-138 uses it.  `in` and `out` may be host or device
 * pointers. */
int glasma_fft3d(glasma_lattice* h, const double* in, double* out, int inverse);
/* The same transform in FP32 (8 planes of complex floats, interleaved re/im), as the gauge fixer
 * runs it with GLASMA_GF_FFT_FP32. */
int glasma_fft3d_f32(glasma_lattice* h, const float* in, float* out, int inverse);

/* Gauss-law violation with no device allocation.  No counterpart in the reference: it exists
 * for callers that cannot call cudaMalloc -- code running while another framework captures a
 * CUDA graph on the stream, memory owned by a pool or arena that forbids outside allocations,
 * real-time loops that must not allocate or synchronise -- and that already hold the fields in
 * device memory.  Same result as glasma_gauss (sync_first = 0) without a lattice handle.
 * Inputs: FP64 device buffers in the library's device layout (S = nx*ny*(nz+2) sites, site
 * s = x + nx*(y + ny*(z+1)), ghost slices included): U[(mu*9 + k)*S + s] complex (k = i + 3*j),
 * E[(mu*8 + a)*S + s], JpStat[a*S + s], JmStat[a*S + s].  Output: result (device, 2 doubles) =
 * {max |G^a|, sqrt(sum G^2 / (8 V))}; zprofile (device, nz doubles, may be NULL).  Work is issued
 * on `stream` (a cudaStream_t, NULL = default stream); the caller synchronises.
 * Scratch is one fixed 512 KiB __device__ array per device, held until the process exits, which
 * limits nz to 992 (larger nz returns GLASMA_ERR_BAD_SHAPE).  The first call on a device looks up
 * that array's address; make it before any stream capture.  The address is cached for the process's
 * lifetime: after a cudaDeviceReset of that device it is stale, so do not call this again after one.
 * All calls on a device share the array: calls that overlap on the GPU race and must be ordered by the
 * caller.  Failures are reported as by every other entry point (status, glasma_last_error()). */
int glasma_gauss_noalloc(const double* U, const double* E, const double* JpStat, const double* JmStat, int nx, int ny,
                         int nz, double ax, double ay, double az, double a_scale, double* result, double* zprofile,
                         void* stream);

/* ---- Adjoint leapfrog, in the lattice's precision (FP64 or FP32 arithmetic and storage; the
 * objective's slice sums are reduced in FP64 either way).  No reference counterpart.
 * Objective on the state after nsteps: L = N(q)/D(q), q = (e0,e1,e2,b0,b1,b2) summed over the slices
 * z in [z_begin, z_end), e_mu = cE_mu sum E_mu^2, b_i = cB_i sum 4 ReTr(1 - P_jk) with the bulk
 * observables' constants (S/OBSERVABLES/BulkObservables.cpp:22-97); N = num.q, D = den.q (D = 1 if
 * den is all zero).  Pressure anisotropy P_L/P_T: num = (1,1,-1,1,1,-1), den = (0,0,1,0,0,1);
 * energy T00: num = (.5,.5,.5,.5,.5,.5), den = 0.
 * glasma_objective evaluates L on the current state.  glasma_adjoint runs nsteps forward from the
 * current state (checkpoints every checkpoint_every steps), evaluates L, and returns dL/d(initial
 * field) for E and the four currents (host buffers in the reference layout, ghost entries zero; any
 * may be NULL), with respect to interior values whose ghost slices are copies of the boundary
 * slices.  Backward pass: time-reversed integration between checkpoints.  The handle is left in
 * its initial state. */
int glasma_objective(glasma_lattice* h, int z_begin, int z_end, const double* num, const double* den, double* value);
int glasma_adjoint(glasma_lattice* h, double dt, int nsteps, int checkpoint_every, int z_begin, int z_end,
                   const double* num, const double* den, double* objective, double* grad_E, double* grad_Jp,
                   double* grad_Jm, double* grad_JpStat, double* grad_JmStat);
const char* glasma_adjoint_last_error(void);

/* ---- Batches of independent events (lattices of uneven sizes) advanced together.
 * No reference counterpart: the reference runs one event per process (seeds are farmed out as
 * separate jobs).  Each event is an ordinary lattice handle (glasma_batch_event gives it, for
 * uploads, downloads and observables); a batch step is one launch per leapfrog kernel over all
 * events' tiles (glasma_batch_set_launch), bit-identical to stepping each event alone.  use_graph != 0 replays
 * blocks of steps (reunitarize_every steps, or 16) from a CUDA graph captured on first use.
 * extents / spacings: 3 values per event. */
typedef struct glasma_batch glasma_batch;
int glasma_batch_create(int n_events, const int* extents, const double* spacings, int precision, int reunitarize_every,
                        glasma_batch** out);
int glasma_batch_destroy(glasma_batch* b);
int glasma_batch_set_stream(glasma_batch* b, void* cuda_stream);
int glasma_batch_event(glasma_batch* b, int event, glasma_lattice** out);
/* Autotunes the electric-field tile once per distinct lattice shape; tiles (may be NULL): n_events ints. */
int glasma_batch_autotune(glasma_batch* b, double dt, int* tiles);
int glasma_batch_step(glasma_batch* b, double dt, int nsteps, int use_graph);
/* Launch shape of the two batch kernels (both cover all events in one launch):
 * GLASMA_BATCH_PERSISTENT — as many blocks as the device holds at once, each walking the tile list;
 * GLASMA_BATCH_TILE_GRID — one block per tile (warps of a block start together on their tile, which
 * keeps the long per-site body in the instruction cache; the default).  Same arithmetic either way. */
#define GLASMA_BATCH_PERSISTENT 0
#define GLASMA_BATCH_TILE_GRID 1
int glasma_batch_set_launch(glasma_batch* b, int mode);
/* Step method of every event of the batch: GLASMA_STEP_TWO_PASS (the staple kernels, the default) or
 * GLASMA_STEP_PLAQUETTE (each event's force summed plaquette by plaquette into its contribution
 * buffer, 48 reals per site, allocated on first use); other methods give GLASMA_ERR_UNSUPPORTED.
 * Either is bit-identical to stepping each event alone with the same method. */
int glasma_batch_set_step_method(glasma_batch* b, int method);
int glasma_batch_get_step_method(glasma_batch* b, int* method);
/* 12-real links for every event of an FP32 batch (see glasma_set_link_storage): the batched step
 * kernels read and write rows 0 and 1 of each link; row 2 is written back at the end of every
 * glasma_batch_step call. */
int glasma_batch_set_link_storage(glasma_batch* b, int reals_per_link);
/* Per-event T00 (volume sum, FP64 reductions), n_events doubles. */
int glasma_batch_energy(glasma_batch* b, double* t00);
int glasma_batch_synchronize(glasma_batch* b);
const char* glasma_batch_last_error(void);

/* Wait for the handle's stream. */
int glasma_synchronize(glasma_lattice* h);
const char* glasma_status_string(int status);
const char* glasma_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* GLASMA_GB300_H */
