/*
 * trv_dropin.hpp -- Triumvirate's C++ estimator interface, served by the
 * GB300 library.
 *
 * Code written against MikeSWang/Triumvirate's C++ headers
 * (src/triumvirate/include/{parameters,particles,dataobjs,threept,
 * twopt}.hpp) compiles against this header and links libtrv_dropin.so
 * (which links libtrvg.so): the classes keep the reference's names,
 * public members and method signatures on the estimator path, and every
 * compute_* function keeps its reference signature.  The definitions
 * (triumvirate_gb300/csrc/dropin/trv_dropin.cpp) convert to the C ABI of
 * trvg.h and run the estimators on the GPU.
 *
 * Differences from the reference:
 *  - ParameterSet has one more member, `precision` ("fp64", the default,
 *    or "fp32mixed"), the arithmetic of meshes and transforms;
 *  - estimators run on CUDA device 0 unless trv::gb300::set_device chose
 *    another (one library context per device and host thread);
 *  - status codes of the library become the reference's exception types
 *    (trv::sys::InvalidParameterError, InvalidDataError,
 *    UnimplementedError); CUDA failures become trv::sys::DeviceError.
 */
#ifndef TRV_DROPIN_HPP_INCLUDED
#define TRV_DROPIN_HPP_INCLUDED

#include <complex>
#include <stdexcept>
#include <string>
#include <vector>

namespace trv {

namespace sys {

/* include/monitor.hpp:683-780 of the reference. */
class InvalidParameterError : public std::invalid_argument {
 public:
  explicit InvalidParameterError(const std::string& msg)
      : std::invalid_argument(msg) {}
};

class InvalidDataError : public std::runtime_error {
 public:
  explicit InvalidDataError(const std::string& msg)
      : std::runtime_error(msg) {}
};

class UnimplementedError : public std::logic_error {
 public:
  explicit UnimplementedError(const std::string& msg)
      : std::logic_error(msg) {}
};

/* A CUDA, cuFFT or device-memory failure (no reference counterpart). */
class DeviceError : public std::runtime_error {
 public:
  explicit DeviceError(const std::string& msg) : std::runtime_error(msg) {}
};

}  // namespace sys

/* include/parameters.hpp:58-290: the members the estimators read, plus
 * `precision`. */
class ParameterSet {
 public:
  std::string catalogue_dir;
  std::string measurement_dir;
  std::string data_catalogue_file;
  std::string rand_catalogue_file;
  std::string catalogue_columns;
  std::string catalogue_dataset;
  std::string output_tag;

  double boxsize[3] = {0., 0., 0.};
  int ngrid[3] = {0, 0, 0};
  double expand = 1.;
  double cutoff_nyq = 0.;
  std::string alignment = "centre";
  std::string padscale = "box";
  double padfactor = 0.;
  std::string assignment = "tsc";
  std::string interlace = "false";

  double volume = 0.;
  long long nmesh = 0;
  int assignment_order = 0;

  std::string catalogue_type;
  std::string statistic_type;
  std::string npoint;
  std::string space;

  int ell1 = 0;
  int ell2 = 0;
  int ELL = 0;
  int i_wa = 0;
  int j_wa = 0;

  std::string form = "diag";
  std::string norm_convention = "particle";
  std::string shape = "diag";

  std::string binning = "lin";
  double bin_min = 0.;
  double bin_max = 0.;
  int num_bins = 0;
  int idx_bin = 0;

  std::string fftw_scheme = "measure";
  std::string use_fftw_wisdom = "false";
  std::string save_binned_vectors = "false";
  int verbose = 20;
  std::string progbar = "false";

  /* GB300 extension: "fp64" or "fp32mixed". */
  std::string precision = "fp64";

  ParameterSet() = default;

  /* The derivations of parameters.cpp:466-1270 on the estimator path:
   * volume, nmesh, assignment_order, npoint and space from
   * statistic_type, shape from form, interlacing off for three-point
   * statistics; throws trv::sys::InvalidParameterError on an invalid
   * value.  Returns 0. */
  int validate(bool init = false);
};

/* include/particles.hpp:62-68. */
struct ParticleData {
  double pos[3];
  double nz;
  double ws;
  double wc;
  double w;
};

/* include/particles.hpp:78-345: particles in host memory, array of
 * structures, as in the reference. */
class ParticleCatalogue {
 public:
  std::string source;
  ParticleData* pdata = nullptr;
  int ntotal = 0;
  double wtotal = 0.;
  double wstotal = 0.;
  double pos_min[3] = {0., 0., 0.};
  double pos_max[3] = {0., 0., 0.};
  double pos_span[3] = {0., 0., 0.};

  explicit ParticleCatalogue(int verbose = -1);
  ~ParticleCatalogue();
  ParticleCatalogue(const ParticleCatalogue&) = delete;
  ParticleCatalogue& operator=(const ParticleCatalogue&) = delete;

  void initialise_particles(const int num);
  void finalise_particles();
  void reset_particles();

  ParticleData& operator[](const int pid);

  /* Text files only ("::" joins sub-files); parsed by the library's
   * multi-threaded reader.  HDF5 files raise InvalidDataError, as a
   * reference build without HDF5 does. */
  int load_catalogue_file(const std::string& catalogue_filepath,
                          const std::string& catalogue_columns,
                          const std::string& catalogue_dataset = "",
                          double volume = 0.);
  int load_particle_data(std::vector<double> x, std::vector<double> y,
                         std::vector<double> z, std::vector<double> nz,
                         std::vector<double> ws, std::vector<double> wc);

  void calc_total_weights();
  void calc_pos_extents(bool init = true);

  void offset_coords(const double dpos[3]);
  void offset_coords_for_periodicity(const double boxsize[3]);

  static void centre_in_box(ParticleCatalogue& catalogue,
                            const double boxsize[3]);
  static void centre_in_box(ParticleCatalogue& catalogue,
                            ParticleCatalogue& catalogue_ref,
                            const double boxsize[3]);
  static void pad_in_box(ParticleCatalogue& catalogue,
                         const double boxsize[3],
                         const double boxsize_pad[3]);
  static void pad_in_box(ParticleCatalogue& catalogue,
                         ParticleCatalogue& catalogue_ref,
                         const double boxsize[3],
                         const double boxsize_pad[3]);
  static void pad_grids(ParticleCatalogue& catalogue,
                        const double boxsize[3], const int ngrid[3],
                        const double ngrid_pad[3]);
  static void pad_grids(ParticleCatalogue& catalogue,
                        ParticleCatalogue& catalogue_ref,
                        const double boxsize[3], const int ngrid[3],
                        const double ngrid_pad[3]);

 private:
  int verbose_ = -1;
};

/* include/dataobjs.hpp:58-158. */
class Binning {
 public:
  std::string space;
  std::string scheme;
  double bin_min = 0.;
  double bin_max = 0.;
  int num_bins = 0;
  std::vector<double> bin_edges;
  std::vector<double> bin_centres;
  std::vector<double> bin_widths;

  explicit Binning(std::string space, std::string scheme);
  explicit Binning(trv::ParameterSet& params);

  void set_bins(double coord_min, double coord_max, int nbin);
  void set_bins();
  void set_bins(double boxsize_max, int ngrid_min);
  void set_bins(std::vector<double> bin_edges);

 private:
  int nbin_pad = 5;
  double dbin_pad_fourier = 1.e-3;
  double dbin_pad_config = 10.;
  void compute_binning();
};

/* include/dataobjs.hpp:186-189. */
struct LineOfSight {
  double pos[3];
};

/* include/dataobjs.hpp:202-283. */
struct PowspecMeasurements {
  int dim = 0;
  std::vector<double> kbin;
  std::vector<double> keff;
  std::vector<int> nmodes;
  std::vector< std::complex<double> > pk_raw;
  std::vector< std::complex<double> > pk_shot;
};

struct BispecMeasurements {
  int dim = 0;
  std::vector<double> k1_bin;
  std::vector<double> k2_bin;
  std::vector<double> k1_eff;
  std::vector<double> k2_eff;
  std::vector<int> nmodes_1;
  std::vector<int> nmodes_2;
  std::vector< std::complex<double> > bk_raw;
  std::vector< std::complex<double> > bk_shot;
};

struct ThreePCFMeasurements {
  int dim = 0;
  std::vector<double> r1_bin;
  std::vector<double> r2_bin;
  std::vector<double> r1_eff;
  std::vector<double> r2_eff;
  std::vector<int> npairs_1;
  std::vector<int> npairs_2;
  std::vector< std::complex<double> > zeta_raw;
  std::vector< std::complex<double> > zeta_shot;
};

struct ThreePCFWindowMeasurements {
  int dim = 0;
  std::vector<double> r1_bin;
  std::vector<double> r2_bin;
  std::vector<double> r1_eff;
  std::vector<double> r2_eff;
  std::vector<int> npairs_1;
  std::vector<int> npairs_2;
  std::vector< std::complex<double> > zeta_raw;
  std::vector< std::complex<double> > zeta_shot;
};

/* include/twopt.hpp:89-104 and include/threept.hpp:138-152. */
double calc_powspec_normalisation_from_particles(ParticleCatalogue& particles,
                                                 double alpha = 1.);
double calc_powspec_normalisation_from_mesh(ParticleCatalogue& particles,
                                            trv::ParameterSet& params,
                                            double alpha = 1.);
double calc_bispec_normalisation_from_particles(ParticleCatalogue& particles,
                                                double alpha = 1.);
double calc_bispec_normalisation_from_mesh(ParticleCatalogue& particles,
                                           trv::ParameterSet& params,
                                           double alpha = 1.);

/* include/twopt.hpp:246-250, 283-287. */
trv::PowspecMeasurements compute_powspec(
    ParticleCatalogue& catalogue_data, ParticleCatalogue& catalogue_rand,
    LineOfSight* los_data, LineOfSight* los_rand, trv::ParameterSet& params,
    trv::Binning& kbinning, double norm_factor);
trv::PowspecMeasurements compute_powspec_in_gpp_box(
    ParticleCatalogue& catalogue_data, trv::ParameterSet& params,
    trv::Binning kbinning, double norm_factor);

/* include/threept.hpp:237-296, 310-314. */
trv::BispecMeasurements compute_bispec(
    ParticleCatalogue& catalogue_data, ParticleCatalogue& catalogue_rand,
    LineOfSight* los_data, LineOfSight* los_rand, trv::ParameterSet& params,
    trv::Binning& kbinning, double norm_factor);
trv::ThreePCFMeasurements compute_3pcf(
    ParticleCatalogue& catalogue_data, ParticleCatalogue& catalogue_rand,
    LineOfSight* los_data, LineOfSight* los_rand, trv::ParameterSet& params,
    trv::Binning& rbinning, double norm_factor);
trv::BispecMeasurements compute_bispec_in_gpp_box(
    ParticleCatalogue& catalogue_data, trv::ParameterSet& params,
    trv::Binning kbinning, double norm_factor);
trv::ThreePCFMeasurements compute_3pcf_in_gpp_box(
    ParticleCatalogue& catalogue_data, trv::ParameterSet& params,
    trv::Binning& rbinning, double norm_factor);
trv::ThreePCFWindowMeasurements compute_3pcf_window(
    ParticleCatalogue& catalogue_rand, LineOfSight* los_rand,
    trv::ParameterSet& params, trv::Binning& rbinning, double alpha,
    double norm_factor, bool wide_angle = false);

namespace gb300 {

/* CUDA device of the estimators called afterwards on this host thread
 * (default 0). */
void set_device(int device);

}  // namespace gb300

}  // namespace trv

#endif  /* TRV_DROPIN_HPP_INCLUDED */
