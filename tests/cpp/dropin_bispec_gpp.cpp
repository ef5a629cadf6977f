// A program written against the reference's C++ interface
// (trv::ParameterSet, trv::ParticleCatalogue, trv::Binning,
// trv::compute_bispec_in_gpp_box; include/threept.hpp:274-278 of
// MikeSWang/Triumvirate), linked with libtrv_dropin.so.  It prepares the
// catalogue as the reference's Python layer does for a periodic box
// (centred, then wrapped), estimates B_000 diag with the reference tests'
// settings (1000 Mpc/h box, 64^3 mesh, TSC, 4 linear bins
// 0.005-0.105 h/Mpc) and prints one row per data-vector entry:
//   k1_bin k1_eff nmodes_1 k2_bin k2_eff nmodes_2 Re(raw) Im(raw)
//   Re(shot) Im(shot)
// Usage: dropin_bispec_gpp CATALOGUE [fp64|fp32mixed]
// A second mode, `dropin_bispec_gpp --errors`, checks that invalid
// parameters raise the reference's exception types.
#include <cstdio>
#include <string>

#include "trv_dropin.hpp"

static int check_errors() {
  trv::ParameterSet p;
  p.boxsize[0] = p.boxsize[1] = p.boxsize[2] = 1000.;
  p.ngrid[0] = p.ngrid[1] = p.ngrid[2] = 32;
  p.assignment = "quartic";
  try {
    p.validate();
    std::printf("no exception for an unknown assignment\n");
    return 1;
  } catch (const trv::sys::InvalidParameterError& e) {
    std::printf("InvalidParameterError: %s\n", e.what());
  }
  trv::ParticleCatalogue empty;
  try {
    trv::calc_bispec_normalisation_from_particles(empty);
    std::printf("no exception for an empty catalogue\n");
    return 1;
  } catch (const trv::sys::InvalidDataError& e) {
    std::printf("InvalidDataError: %s\n", e.what());
  }
  return 0;
}

int main(int argc, char** argv) {
  if (argc >= 2 && std::string(argv[1]) == "--errors") return check_errors();
  if (argc < 2) {
    std::fprintf(stderr, "usage: %s CATALOGUE [fp64|fp32mixed]\n", argv[0]);
    return 2;
  }
  trv::ParameterSet params;
  for (int a = 0; a < 3; ++a) {
    params.boxsize[a] = 1000.;
    params.ngrid[a] = 64;
  }
  params.assignment = "tsc";
  params.interlace = "false";
  params.statistic_type = "bispec";
  params.ell1 = params.ell2 = params.ELL = 0;
  params.form = "diag";
  params.binning = "lin";
  params.bin_min = 0.005;
  params.bin_max = 0.105;
  params.num_bins = 4;
  params.verbose = 0;
  params.precision = argc >= 3 ? argv[2] : "fp64";
  try {
    params.validate();
    trv::ParticleCatalogue cat;
    cat.load_catalogue_file(argv[1], "x,y,z,nz", "", params.volume);
    trv::ParticleCatalogue::centre_in_box(cat, params.boxsize);
    cat.offset_coords_for_periodicity(params.boxsize);
    trv::Binning kbinning(params);
    kbinning.set_bins();
    const double norm = trv::calc_bispec_normalisation_from_particles(cat);
    trv::BispecMeasurements m =
        trv::compute_bispec_in_gpp_box(cat, params, kbinning, norm);
    for (int i = 0; i < m.dim; ++i)
      std::printf("%.17g %.17g %d %.17g %.17g %d %.17g %.17g %.17g %.17g\n",
                  m.k1_bin[i], m.k1_eff[i], m.nmodes_1[i], m.k2_bin[i],
                  m.k2_eff[i], m.nmodes_2[i], m.bk_raw[i].real(),
                  m.bk_raw[i].imag(), m.bk_shot[i].real(),
                  m.bk_shot[i].imag());
  } catch (const std::exception& e) {
    std::fprintf(stderr, "error: %s\n", e.what());
    return 1;
  }
  return 0;
}
