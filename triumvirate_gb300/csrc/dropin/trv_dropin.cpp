// Definitions of the reference's C++ estimator interface (trv_dropin.hpp)
// over the C ABI of the GB300 library (trvg.h).
//
// Catalogue bookkeeping (extents, totals, offsets, centring, padding,
// periodic wrapping) follows particles.cpp:552-888 of MikeSWang/Triumvirate
// operation for operation on the host, so that coordinates are the same
// doubles the reference would hand its estimators; the estimators
// themselves, the mesh normalisations and file parsing run in the library.
#include "trv_dropin.hpp"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <map>
#include <memory>
#include <utility>

#include "trvg.h"

namespace trv {

namespace {

[[noreturn]] void raise_status(int status) {
  const std::string msg = trvg_last_error();
  switch (status) {
    case TRVG_ERR_INVALID_PARAMETER:
      throw sys::InvalidParameterError(msg);
    case TRVG_ERR_INVALID_DATA:
      throw sys::InvalidDataError(msg);
    case TRVG_ERR_UNIMPLEMENTED:
      throw sys::UnimplementedError(msg);
    default:
      throw sys::DeviceError(msg);
  }
}

void check(int status) {
  if (status != TRVG_OK) raise_status(status);
}

// One library context per (host thread, device): a context's calls must
// not overlap, and the reference's functions take no context argument.
thread_local int t_device = 0;

struct ContextDeleter {
  void operator()(trvg_context* c) const {
    if (c != nullptr) trvg_context_destroy(c);
  }
};

trvg_context* context() {
  thread_local std::map<int, std::unique_ptr<trvg_context, ContextDeleter>>
      contexts;
  auto it = contexts.find(t_device);
  if (it == contexts.end()) {
    trvg_context* c = nullptr;
    check(trvg_context_create(t_device, &c));
    it = contexts.emplace(t_device,
                          std::unique_ptr<trvg_context, ContextDeleter>(c))
             .first;
  }
  return it->second.get();
}

int order_of(const std::string& assignment) {
  if (assignment == "ngp") return 1;
  if (assignment == "cic") return 2;
  if (assignment == "tsc") return 3;
  if (assignment == "pcs") return 4;
  throw sys::InvalidParameterError(
      "Mesh assignment scheme must be 'ngp', 'cic', 'tsc' or 'pcs': "
      "`assignment` = '" + assignment + "'.");
}

int shape_of(const std::string& shape) {
  if (shape == "diag") return TRVG_SHAPE_DIAG;
  if (shape == "off-diag") return TRVG_SHAPE_OFFDIAG;
  if (shape == "row") return TRVG_SHAPE_ROW;
  if (shape == "full") return TRVG_SHAPE_FULL;
  if (shape == "triu") return TRVG_SHAPE_TRIU;
  throw sys::InvalidParameterError("Three-point statistic form is not "
                                   "recognised: `shape` = '" + shape + "'.");
}

// The C-ABI parameter block of a validated parameter set.
trvg_params c_params(const ParameterSet& p) {
  trvg_params c{};
  for (int a = 0; a < 3; ++a) {
    c.boxsize[a] = p.boxsize[a];
    c.ngrid[a] = p.ngrid[a];
  }
  c.assignment_order = order_of(p.assignment);
  c.interlace = p.interlace == "true" ? 1 : 0;
  c.ell1 = p.ell1;
  c.ell2 = p.ell2;
  c.ELL = p.ELL;
  c.shape = shape_of(p.shape);
  c.idx_bin = p.idx_bin;
  if (p.precision == "fp64") {
    c.precision = TRVG_PREC_FP64;
  } else if (p.precision == "fp32mixed") {
    c.precision = TRVG_PREC_FP32_MIXED;
  } else {
    throw sys::InvalidParameterError(
        "`precision` must be 'fp64' or 'fp32mixed': '" + p.precision + "'.");
  }
  c.verbose = p.verbose;
  c.i_wa = p.i_wa;
  c.j_wa = p.j_wa;
  return c;
}

// Structure-of-arrays host copy of a catalogue (and its lines of sight).
struct Columns {
  std::vector<double> x, y, z, w, lx, ly, lz;
  trvg_catalogue c{};

  Columns(ParticleCatalogue& cat, const LineOfSight* los) {
    if (cat.pdata == nullptr)
      throw sys::InvalidDataError("Particle data are uninitialised.");
    const size_t n = size_t(cat.ntotal);
    x.resize(n);
    y.resize(n);
    z.resize(n);
    w.resize(n);
    for (size_t i = 0; i < n; ++i) {
      x[i] = cat.pdata[i].pos[0];
      y[i] = cat.pdata[i].pos[1];
      z[i] = cat.pdata[i].pos[2];
      w[i] = cat.pdata[i].w;
    }
    c.n = int64_t(n);
    c.x = x.data();
    c.y = y.data();
    c.z = z.data();
    c.w = w.data();
    c.memory = TRVG_MEM_HOST;
    if (los != nullptr) {
      lx.resize(n);
      ly.resize(n);
      lz.resize(n);
      for (size_t i = 0; i < n; ++i) {
        lx[i] = los[i].pos[0];
        ly[i] = los[i].pos[1];
        lz[i] = los[i].pos[2];
      }
      c.los_x = lx.data();
      c.los_y = ly.data();
      c.los_z = lz.data();
    }
  }
};

trvg_binning c_binning(const Binning& b) {
  if (b.num_bins <= 0 || b.bin_edges.size() != size_t(b.num_bins) + 1 ||
      b.bin_centres.size() != size_t(b.num_bins))
    throw sys::InvalidParameterError("Binning has no bins set.");
  trvg_binning c{};
  c.num_bins = b.num_bins;
  c.bin_edges = b.bin_edges.data();
  c.bin_centres = b.bin_centres.data();
  return c;
}

// Host buffers of a three-point data vector and their C-ABI view.
struct ThreeptBuffers {
  int dim = 0;
  std::vector<double> c1, e1, c2, e2, raw, shot;
  std::vector<int32_t> n1, n2;
  trvg_threept_out out{};

  ThreeptBuffers(const ParameterSet& p, int num_bins) {
    check(trvg_data_vector_dim(shape_of(p.shape), num_bins, p.idx_bin,
                               &dim));
    c1.resize(dim);
    e1.resize(dim);
    c2.resize(dim);
    e2.resize(dim);
    raw.resize(2 * size_t(dim));
    shot.resize(2 * size_t(dim));
    n1.resize(dim);
    n2.resize(dim);
    out.dim = dim;
    out.coord1_bin = c1.data();
    out.coord1_eff = e1.data();
    out.count_1 = n1.data();
    out.coord2_bin = c2.data();
    out.coord2_eff = e2.data();
    out.count_2 = n2.data();
    out.raw = raw.data();
    out.shot = shot.data();
  }

  template <class M>
  void fill_bispec(M& m) const {
    m.dim = dim;
    m.k1_bin = c1;
    m.k1_eff = e1;
    m.k2_bin = c2;
    m.k2_eff = e2;
    m.nmodes_1.assign(n1.begin(), n1.end());
    m.nmodes_2.assign(n2.begin(), n2.end());
    m.bk_raw = complex_of(raw);
    m.bk_shot = complex_of(shot);
  }

  template <class M>
  void fill_3pcf(M& m) const {
    m.dim = dim;
    m.r1_bin = c1;
    m.r1_eff = e1;
    m.r2_bin = c2;
    m.r2_eff = e2;
    m.npairs_1.assign(n1.begin(), n1.end());
    m.npairs_2.assign(n2.begin(), n2.end());
    m.zeta_raw = complex_of(raw);
    m.zeta_shot = complex_of(shot);
  }

  static std::vector<std::complex<double>> complex_of(
      const std::vector<double>& v) {
    std::vector<std::complex<double>> out(v.size() / 2);
    for (size_t i = 0; i < out.size(); ++i)
      out[i] = std::complex<double>(v[2 * i], v[2 * i + 1]);
    return out;
  }
};

// alpha = wstotal_data / wstotal_rand (threept.cpp:271, twopt.cpp:266).
double alpha_of(const ParticleCatalogue& d, const ParticleCatalogue& r) {
  return d.wstotal / r.wstotal;
}

// sum ws nz^(order - 1) wc^order, the particle normalisation's
// denominator (twopt.cpp:56-99, threept.cpp:96-136).
double particle_norm_sum(ParticleCatalogue& particles, int order) {
  if (particles.pdata == nullptr)
    throw sys::InvalidDataError("Particle data are uninitialised.");
  double norm = 0.;
  for (int pid = 0; pid < particles.ntotal; ++pid) {
    const ParticleData& q = particles.pdata[pid];
    norm += q.ws * std::pow(q.nz, order - 1) * std::pow(q.wc, order);
  }
  if (norm == 0.)
    throw sys::InvalidDataError(
        "Particle 'nz' values appear to be all zeros. Check the input "
        "catalogue contains valid 'nz' field.");
  return norm;
}

double mesh_norm(ParticleCatalogue& particles, ParameterSet& params,
                 int order) {
  Columns cols(particles, nullptr);
  const trvg_params c = c_params(params);
  double norm = 0.;
  check(trvg_calc_grid_based_powlaw_norm(context(), &c, &cols.c, order,
                                         &norm));
  return norm;
}

}  // namespace

// ---------------------------------------------------------------------------
// ParameterSet (parameters.cpp:466-1270, on-path derivations)
// ---------------------------------------------------------------------------

int ParameterSet::validate(bool /*init*/) {
  for (int a = 0; a < 3; ++a) {
    if (!(boxsize[a] > 0.))
      throw sys::InvalidParameterError(
          "Box size must be positive in every dimension.");
    if (ngrid[a] <= 0)
      throw sys::InvalidParameterError(
          "Mesh number must be positive in every dimension.");
  }
  volume = boxsize[0] * boxsize[1] * boxsize[2];
  nmesh = (long long)ngrid[0] * ngrid[1] * ngrid[2];
  assignment_order = order_of(assignment);
  if (interlace == "true" || interlace == "on") {
    interlace = "true";
  } else if (interlace == "false" || interlace == "off") {
    interlace = "false";
  } else {
    throw sys::InvalidParameterError(
        "Interlacing must be 'true'/'on' or 'false'/'off': `interlace` = '" +
        interlace + "'.");
  }
  static const std::map<std::string, std::pair<const char*, const char*>>
      kStat = {{"powspec", {"2pt", "fourier"}},
               {"2pcf", {"2pt", "config"}},
               {"2pcf-win", {"2pt", "config"}},
               {"bispec", {"3pt", "fourier"}},
               {"3pcf", {"3pt", "config"}},
               {"3pcf-win", {"3pt", "config"}},
               {"3pcf-win-wa", {"3pt", "config"}},
               {"modes", {"none", "fourier"}},
               {"pairs", {"none", "config"}}};
  if (!statistic_type.empty()) {
    auto it = kStat.find(statistic_type);
    if (it == kStat.end())
      throw sys::InvalidParameterError(
          "Statistic type is not recognised: `statistic_type` = '" +
          statistic_type + "'.");
    npoint = it->second.first;
    space = it->second.second;
  }
  if (form != "full" && form != "diag" && form != "off-diag" &&
      form != "row")
    throw sys::InvalidParameterError(
        "Three-point statistic form is not recognised: `form` = '" + form +
        "'.");
  shape = (form == "full" && ell1 == ell2) ? "triu" : form;
  if (norm_convention != "none" && norm_convention != "particle" &&
      norm_convention != "mesh" && norm_convention != "mesh-mixed")
    throw sys::InvalidParameterError(
        "Normalisation convention must be 'none', 'particle', 'mesh' or "
        "'mesh-mixed': `norm_convention` = '" + norm_convention + "'.");
  if (num_bins > 0 && (idx_bin >= num_bins || idx_bin <= -num_bins))
    throw sys::InvalidParameterError(
        "Bin index `idx_bin` must be < `num_bins` in absolute value.");
  if (npoint == "3pt" && interlace == "true") interlace = "false";
  if (precision != "fp64" && precision != "fp32mixed")
    throw sys::InvalidParameterError(
        "`precision` must be 'fp64' or 'fp32mixed': '" + precision + "'.");
  return 0;
}

// ---------------------------------------------------------------------------
// ParticleCatalogue (particles.cpp:36-888)
// ---------------------------------------------------------------------------

ParticleCatalogue::ParticleCatalogue(int verbose) : verbose_(verbose) {}

ParticleCatalogue::~ParticleCatalogue() { finalise_particles(); }

void ParticleCatalogue::initialise_particles(const int num) {
  if (num <= 0)
    throw sys::InvalidParameterError("Number of particles is non-positive.");
  ntotal = num;
  reset_particles();
  pdata = new ParticleData[size_t(num)];
}

void ParticleCatalogue::finalise_particles() { reset_particles(); }

void ParticleCatalogue::reset_particles() {
  delete[] pdata;
  pdata = nullptr;
}

ParticleData& ParticleCatalogue::operator[](const int pid) {
  return pdata[pid];
}

int ParticleCatalogue::load_catalogue_file(
    const std::string& catalogue_filepath,
    const std::string& catalogue_columns,
    const std::string& /*catalogue_dataset*/, double volume) {
  source = "extfile:" + catalogue_filepath;
  trvg_dcat* dc = nullptr;
  check(trvg_dcat_read_text(context(), catalogue_filepath.c_str(),
                            catalogue_columns.c_str(), volume, &dc));
  std::unique_ptr<trvg_dcat, int (*)(trvg_dcat*)> hold(dc, trvg_dcat_destroy);
  int64_t n = 0;
  check(trvg_dcat_info(context(), dc, &n, nullptr, nullptr, nullptr,
                       nullptr));
  if (n <= 0)
    throw sys::InvalidDataError("Catalogue file has no particles: " +
                                catalogue_filepath);
  if (n > int64_t(2147483647))
    throw sys::InvalidDataError(
        "Catalogue has more particles than an int counts.");
  const char* names[6] = {"x", "y", "z", "nz", "ws", "wc"};
  std::vector<double> cols[6];
  for (int c = 0; c < 6; ++c) {
    cols[c].resize(size_t(n));
    check(trvg_dcat_download(context(), dc, names[c], cols[c].data()));
  }
  const std::string keep = source;
  load_particle_data(std::move(cols[0]), std::move(cols[1]),
                     std::move(cols[2]), std::move(cols[3]),
                     std::move(cols[4]), std::move(cols[5]));
  source = keep;
  return 0;
}

int ParticleCatalogue::load_particle_data(std::vector<double> x,
                                          std::vector<double> y,
                                          std::vector<double> z,
                                          std::vector<double> nz,
                                          std::vector<double> ws,
                                          std::vector<double> wc) {
  source = "extdata";
  const size_t n = x.size();
  if (y.size() != n || z.size() != n || nz.size() != n || ws.size() != n ||
      wc.size() != n)
    throw sys::InvalidDataError(
        "Inconsistent particle data dimensions (source=extdata).");
  initialise_particles(int(n));
  for (size_t i = 0; i < n; ++i) {
    ParticleData& q = pdata[i];
    q.pos[0] = x[i];
    q.pos[1] = y[i];
    q.pos[2] = z[i];
    q.nz = nz[i];
    q.ws = ws[i];
    q.wc = wc[i];
    q.w = ws[i] * wc[i];
  }
  calc_total_weights();
  calc_pos_extents();
  return 0;
}

void ParticleCatalogue::calc_total_weights() {
  if (pdata == nullptr)
    throw sys::InvalidDataError("Particle data are uninitialised.");
  double wt = 0., wst = 0.;
  for (int pid = 0; pid < ntotal; ++pid) {
    wt += pdata[pid].w;
    wst += pdata[pid].ws;
  }
  wtotal = wt;
  wstotal = wst;
}

void ParticleCatalogue::calc_pos_extents(bool /*init*/) {
  if (pdata == nullptr)
    throw sys::InvalidDataError("Particle data are uninitialised.");
  double lo[3], hi[3];
  for (int a = 0; a < 3; ++a) lo[a] = hi[a] = pdata[0].pos[a];
  for (int pid = 0; pid < ntotal; ++pid)
    for (int a = 0; a < 3; ++a) {
      const double v = pdata[pid].pos[a];
      lo[a] = lo[a] < v ? lo[a] : v;
      hi[a] = hi[a] > v ? hi[a] : v;
    }
  for (int a = 0; a < 3; ++a) {
    pos_min[a] = lo[a];
    pos_max[a] = hi[a];
    pos_span[a] = hi[a] - lo[a];
  }
}

void ParticleCatalogue::offset_coords(const double dpos[3]) {
  if (pdata == nullptr)
    throw sys::InvalidDataError("Particle data are uninitialised.");
  for (int pid = 0; pid < ntotal; ++pid)
    for (int a = 0; a < 3; ++a) pdata[pid].pos[a] -= dpos[a];
  calc_pos_extents();
}

void ParticleCatalogue::offset_coords_for_periodicity(
    const double boxsize[3]) {
  for (int pid = 0; pid < ntotal; ++pid)
    for (int a = 0; a < 3; ++a) {
      double& v = pdata[pid].pos[a];
      if (v >= boxsize[a]) {
        v = std::fmod(v, boxsize[a]);
      } else if (v < 0.) {
        v = std::fmod(v, boxsize[a]) + boxsize[a];
      }
    }
  calc_pos_extents();
}

namespace {

// The offset that moves the mid-point of ref's extents to the box centre.
void centre_offset(ParticleCatalogue& ref, const double boxsize[3],
                   double dvec[3]) {
  ref.calc_pos_extents(false);
  for (int a = 0; a < 3; ++a)
    dvec[a] = (ref.pos_min[a] + ref.pos_max[a]) / 2. - boxsize[a] / 2.;
}

}  // namespace

void ParticleCatalogue::centre_in_box(ParticleCatalogue& catalogue,
                                      const double boxsize[3]) {
  double dvec[3];
  centre_offset(catalogue, boxsize, dvec);
  catalogue.offset_coords(dvec);
}

void ParticleCatalogue::centre_in_box(ParticleCatalogue& catalogue,
                                      ParticleCatalogue& catalogue_ref,
                                      const double boxsize[3]) {
  catalogue.calc_pos_extents(false);
  double dvec[3];
  centre_offset(catalogue_ref, boxsize, dvec);
  catalogue_ref.offset_coords(dvec);
  catalogue.offset_coords(dvec);
}

void ParticleCatalogue::pad_in_box(ParticleCatalogue& catalogue,
                                   const double boxsize[3],
                                   const double boxsize_pad[3]) {
  catalogue.calc_pos_extents(false);
  double dvec[3];
  for (int a = 0; a < 3; ++a)
    dvec[a] = catalogue.pos_min[a] - boxsize_pad[a] * boxsize[a];
  catalogue.offset_coords(dvec);
}

void ParticleCatalogue::pad_in_box(ParticleCatalogue& catalogue,
                                   ParticleCatalogue& catalogue_ref,
                                   const double boxsize[3],
                                   const double boxsize_pad[3]) {
  catalogue.calc_pos_extents(false);
  catalogue_ref.calc_pos_extents(false);
  double dvec[3];
  for (int a = 0; a < 3; ++a)
    dvec[a] = catalogue_ref.pos_min[a] - boxsize_pad[a] * boxsize[a];
  catalogue_ref.offset_coords(dvec);
  catalogue.offset_coords(dvec);
}

void ParticleCatalogue::pad_grids(ParticleCatalogue& catalogue,
                                  const double boxsize[3], const int ngrid[3],
                                  const double ngrid_pad[3]) {
  catalogue.calc_pos_extents(false);
  double dvec[3];
  for (int a = 0; a < 3; ++a) {
    dvec[a] = catalogue.pos_min[a];
    dvec[a] -= ngrid_pad[a] * boxsize[a] / double(ngrid[a]);
  }
  catalogue.offset_coords(dvec);
}

void ParticleCatalogue::pad_grids(ParticleCatalogue& catalogue,
                                  ParticleCatalogue& catalogue_ref,
                                  const double boxsize[3], const int ngrid[3],
                                  const double ngrid_pad[3]) {
  catalogue_ref.calc_pos_extents(false);
  double dvec[3];
  for (int a = 0; a < 3; ++a)
    dvec[a] = catalogue_ref.pos_min[a] -
              ngrid_pad[a] * boxsize[a] / double(ngrid[a]);
  catalogue_ref.offset_coords(dvec);
  catalogue.offset_coords(dvec);
}

// ---------------------------------------------------------------------------
// Binning (dataobjs.cpp:39-266)
// ---------------------------------------------------------------------------

Binning::Binning(std::string space_, std::string scheme_)
    : space(std::move(space_)), scheme(std::move(scheme_)) {
  if (space != "fourier" && space != "config")
    throw sys::InvalidParameterError("Unrecognised coordinate space: '" +
                                     space + "'.");
}

Binning::Binning(ParameterSet& params)
    : Binning(params.space, params.binning) {
  bin_min = params.bin_min;
  bin_max = params.bin_max;
  num_bins = params.num_bins;
}

void Binning::set_bins(double coord_min, double coord_max, int nbin) {
  if (coord_min < 0.)
    throw sys::InvalidParameterError("Bin range must be non-negative.");
  if (nbin <= 0)
    throw sys::InvalidParameterError("Number of bins must be positive.");
  bin_min = coord_min;
  bin_max = coord_max;
  num_bins = nbin;
  compute_binning();
}

void Binning::set_bins() { set_bins(bin_min, bin_max, num_bins); }

void Binning::set_bins(double boxsize_max, int ngrid_min) {
  scheme = "lin";
  bin_min = 0.;
  double width;
  if (space == "config") {
    width = boxsize_max / double(ngrid_min);
    bin_max = boxsize_max / 2.;
  } else {
    width = 2. * M_PI / boxsize_max;
    bin_max = M_PI * double(ngrid_min) / boxsize_max;
  }
  bin_max += width / 2.;
  num_bins = ngrid_min / 2;
  compute_binning();
}

void Binning::set_bins(std::vector<double> edges) {
  if (edges.size() < 2)
    throw sys::InvalidParameterError("Custom binning needs >= 2 edges.");
  scheme = "custom";
  bin_min = edges.front();
  bin_max = edges.back();
  num_bins = int(edges.size()) - 1;
  bin_edges = edges;
  bin_centres.resize(num_bins);
  bin_widths.resize(num_bins);
  for (int i = 0; i < num_bins; ++i) {
    bin_centres[i] = (edges[i] + edges[i + 1]) / 2.;
    bin_widths[i] = edges[i + 1] - edges[i];
  }
}

void Binning::compute_binning() {
  bin_edges.clear();
  bin_centres.clear();
  bin_widths.clear();
  const double pad = space == "fourier" ? dbin_pad_fourier : dbin_pad_config;
  auto push = [&](double left, double centre, double width) {
    bin_edges.push_back(left);
    bin_centres.push_back(centre);
    bin_widths.push_back(width);
  };
  if (scheme == "lin") {
    const double d = (bin_max - bin_min) / double(num_bins);
    for (int i = 0; i < num_bins; ++i) {
      const double left = bin_min + d * i;
      push(left, left + d / 2., d);
    }
  } else if (scheme == "log") {
    if (bin_min == 0.)
      throw sys::InvalidParameterError(
          "Cannot use logarithmic binning when the lowest edge is zero.");
    const double dln = (std::log(bin_max) - std::log(bin_min)) /
                       double(num_bins);
    for (int i = 0; i < num_bins; ++i) {
      const double left = bin_min * std::exp(dln * i);
      const double right = bin_min * std::exp(dln * (i + 1));
      push(left, (left + right) / 2., right - left);
    }
  } else if (scheme == "linpad" || scheme == "logpad") {
    for (int i = 0; i < nbin_pad; ++i) {
      const double left = pad * i;
      push(left, left + pad / 2., pad);
    }
    const double start = pad * nbin_pad;
    if (scheme == "linpad") {
      const double d = (bin_max - start) / double(num_bins - nbin_pad);
      for (int i = nbin_pad; i < num_bins; ++i) {
        const double left = start + d * (i - nbin_pad);
        push(left, left + d / 2., d);
      }
    } else {
      const double dln = (std::log(bin_max) - std::log(start)) /
                         double(num_bins - nbin_pad);
      for (int i = nbin_pad; i < num_bins; ++i) {
        const double left = start * std::exp(dln * (i - nbin_pad));
        const double right = start * std::exp(dln * (i - nbin_pad + 1));
        push(left, (left + right) / 2., right - left);
      }
    }
  } else {
    throw sys::InvalidParameterError(
        "Unrecognised/unsupported binning `scheme`: '" + scheme + "'.");
  }
  bin_edges.push_back(bin_max);
}

// ---------------------------------------------------------------------------
// Normalisations (twopt.cpp:56-110, threept.cpp:96-149)
// ---------------------------------------------------------------------------

double calc_powspec_normalisation_from_particles(ParticleCatalogue& particles,
                                                 double alpha) {
  return 1. / (alpha * particle_norm_sum(particles, 2));
}

double calc_powspec_normalisation_from_mesh(ParticleCatalogue& particles,
                                            ParameterSet& params,
                                            double alpha) {
  return mesh_norm(particles, params, 2) / std::pow(alpha, 2);
}

double calc_bispec_normalisation_from_particles(ParticleCatalogue& particles,
                                                double alpha) {
  return 1. / (alpha * particle_norm_sum(particles, 3));
}

double calc_bispec_normalisation_from_mesh(ParticleCatalogue& particles,
                                           ParameterSet& params,
                                           double alpha) {
  return mesh_norm(particles, params, 3) / std::pow(alpha, 3);
}

// ---------------------------------------------------------------------------
// Estimators
// ---------------------------------------------------------------------------

PowspecMeasurements compute_powspec(ParticleCatalogue& catalogue_data,
                                    ParticleCatalogue& catalogue_rand,
                                    LineOfSight* los_data,
                                    LineOfSight* los_rand,
                                    ParameterSet& params,
                                    Binning& kbinning, double norm_factor) {
  Columns d(catalogue_data, los_data), r(catalogue_rand, los_rand);
  const trvg_params c = c_params(params);
  const trvg_binning b = c_binning(kbinning);
  PowspecMeasurements m;
  m.dim = b.num_bins;
  std::vector<double> raw(2 * size_t(m.dim)), shot(2 * size_t(m.dim));
  std::vector<int32_t> nm(m.dim);
  m.kbin.resize(m.dim);
  m.keff.resize(m.dim);
  trvg_powspec_out o{m.dim, m.kbin.data(), m.keff.data(), nm.data(),
                     raw.data(), shot.data()};
  check(trvg_compute_powspec(context(), &c, &d.c, &r.c,
                             alpha_of(catalogue_data, catalogue_rand), &b,
                             norm_factor, &o));
  m.nmodes.assign(nm.begin(), nm.end());
  m.pk_raw = ThreeptBuffers::complex_of(raw);
  m.pk_shot = ThreeptBuffers::complex_of(shot);
  return m;
}

PowspecMeasurements compute_powspec_in_gpp_box(
    ParticleCatalogue& catalogue_data, ParameterSet& params,
    Binning kbinning, double norm_factor) {
  Columns d(catalogue_data, nullptr);
  const trvg_params c = c_params(params);
  const trvg_binning b = c_binning(kbinning);
  PowspecMeasurements m;
  m.dim = b.num_bins;
  std::vector<double> raw(2 * size_t(m.dim)), shot(2 * size_t(m.dim));
  std::vector<int32_t> nm(m.dim);
  m.kbin.resize(m.dim);
  m.keff.resize(m.dim);
  trvg_powspec_out o{m.dim, m.kbin.data(), m.keff.data(), nm.data(),
                     raw.data(), shot.data()};
  check(trvg_compute_powspec_in_gpp_box(context(), &c, &d.c, &b, norm_factor,
                                        &o));
  m.nmodes.assign(nm.begin(), nm.end());
  m.pk_raw = ThreeptBuffers::complex_of(raw);
  m.pk_shot = ThreeptBuffers::complex_of(shot);
  return m;
}

BispecMeasurements compute_bispec(ParticleCatalogue& catalogue_data,
                                  ParticleCatalogue& catalogue_rand,
                                  LineOfSight* los_data,
                                  LineOfSight* los_rand, ParameterSet& params,
                                  Binning& kbinning, double norm_factor) {
  Columns d(catalogue_data, los_data), r(catalogue_rand, los_rand);
  const trvg_params c = c_params(params);
  const trvg_binning b = c_binning(kbinning);
  ThreeptBuffers buf(params, b.num_bins);
  check(trvg_compute_bispec(context(), &c, &d.c, &r.c,
                            alpha_of(catalogue_data, catalogue_rand), &b,
                            norm_factor, &buf.out));
  BispecMeasurements m;
  buf.fill_bispec(m);
  return m;
}

ThreePCFMeasurements compute_3pcf(ParticleCatalogue& catalogue_data,
                                  ParticleCatalogue& catalogue_rand,
                                  LineOfSight* los_data,
                                  LineOfSight* los_rand, ParameterSet& params,
                                  Binning& rbinning, double norm_factor) {
  Columns d(catalogue_data, los_data), r(catalogue_rand, los_rand);
  const trvg_params c = c_params(params);
  const trvg_binning b = c_binning(rbinning);
  ThreeptBuffers buf(params, b.num_bins);
  check(trvg_compute_3pcf(context(), &c, &d.c, &r.c,
                          alpha_of(catalogue_data, catalogue_rand), &b,
                          norm_factor, &buf.out));
  ThreePCFMeasurements m;
  buf.fill_3pcf(m);
  return m;
}

BispecMeasurements compute_bispec_in_gpp_box(ParticleCatalogue& catalogue_data,
                                             ParameterSet& params,
                                             Binning kbinning,
                                             double norm_factor) {
  Columns d(catalogue_data, nullptr);
  const trvg_params c = c_params(params);
  const trvg_binning b = c_binning(kbinning);
  ThreeptBuffers buf(params, b.num_bins);
  check(trvg_compute_bispec_in_gpp_box(context(), &c, &d.c, &b, norm_factor,
                                       &buf.out));
  BispecMeasurements m;
  buf.fill_bispec(m);
  return m;
}

ThreePCFMeasurements compute_3pcf_in_gpp_box(ParticleCatalogue& catalogue_data,
                                             ParameterSet& params,
                                             Binning& rbinning,
                                             double norm_factor) {
  Columns d(catalogue_data, nullptr);
  const trvg_params c = c_params(params);
  const trvg_binning b = c_binning(rbinning);
  ThreeptBuffers buf(params, b.num_bins);
  check(trvg_compute_3pcf_in_gpp_box(context(), &c, &d.c, &b, norm_factor,
                                     &buf.out));
  ThreePCFMeasurements m;
  buf.fill_3pcf(m);
  return m;
}

ThreePCFWindowMeasurements compute_3pcf_window(
    ParticleCatalogue& catalogue_rand, LineOfSight* los_rand,
    ParameterSet& params, Binning& rbinning, double alpha,
    double norm_factor, bool wide_angle) {
  Columns r(catalogue_rand, los_rand);
  const trvg_params c = c_params(params);
  const trvg_binning b = c_binning(rbinning);
  ThreeptBuffers buf(params, b.num_bins);
  check(trvg_compute_3pcf_window(context(), &c, &r.c, alpha, &b, norm_factor,
                                 wide_angle ? 1 : 0, &buf.out));
  ThreePCFWindowMeasurements m;
  buf.fill_3pcf(m);
  return m;
}

namespace gb300 {

void set_device(int device) { t_device = device; }

}  // namespace gb300

}  // namespace trv
