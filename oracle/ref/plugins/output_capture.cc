// Capture output plugin, registered into the reference's own plugin map
// (output_plugin_creator_concrete, include/output_plugin.hh:110-124): writes
// what ic_generator::run hands to an output plugin -- the particle container
// (positions, velocities, IDs, masses) or the Lagrangian field grids -- as
// .npy arrays into the directory [output] filename, together with the
// cosmology scalars the run used (scalars.txt).  Test infrastructure for
// oracle/_ref.
//
//   [output] format = capture, filename = <dir>
//            capture_type = particles | field_lagrangian | field_eulerian
//            capture_type_baryon (default capture_type)
//            capture_64bit_reals, capture_64bit_ids (default yes)
//            capture_lunit, capture_vunit (default BoxLength), capture_munit (1)
#include <sys/stat.h>
#include <sys/types.h>

#include <cstdint>
#include <cstdio>
#include <fstream>
#include <iomanip>
#include <string>
#include <vector>

#include <general.hh>
#include <output_plugin.hh>

namespace {

// minimal .npy (version 1.0) writer, C order, little endian
void write_npy(const std::string& path, const void* data, size_t count, const char* descr,
               const std::vector<size_t>& shape) {
  std::string sh = "(";
  for (size_t i = 0; i < shape.size(); ++i) sh += std::to_string(shape[i]) + (shape.size() == 1 ? "," : (i + 1 < shape.size() ? ", " : ""));
  sh += ")";
  std::string hdr = std::string("{'descr': '") + descr + "', 'fortran_order': False, 'shape': " + sh + ", }";
  const size_t total = 10 + hdr.size() + 1;
  hdr.append((64 - total % 64) % 64, ' ');
  hdr += '\n';
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) throw std::runtime_error("capture: cannot write " + path);
  const unsigned char magic[8] = {0x93, 'N', 'U', 'M', 'P', 'Y', 1, 0};
  std::fwrite(magic, 1, 8, f);
  const uint16_t hl = (uint16_t)hdr.size();
  std::fwrite(&hl, 2, 1, f);
  std::fwrite(hdr.data(), 1, hdr.size(), f);
  size_t esz = (descr[2] == '8') ? 8 : 4;
  std::fwrite(data, esz, count, f);
  std::fclose(f);
}

std::string species_name(const cosmo_species& s) {
  return s == cosmo_species::dm ? "dm" : (s == cosmo_species::baryon ? "baryon" : "neutrino");
}

std::string component_name(const fluid_component& c) {
  switch (c) {
    case fluid_component::density: return "density";
    case fluid_component::vx: return "vx";
    case fluid_component::vy: return "vy";
    case fluid_component::vz: return "vz";
    case fluid_component::dx: return "dx";
    case fluid_component::dy: return "dy";
    case fluid_component::dz: return "dz";
    case fluid_component::mass: return "mass";
  }
  return "unknown";
}

class capture_output_plugin : public output_plugin {
  output_type type_, type_baryon_;
  bool real64_, id64_;
  double lunit_, vunit_, munit_;

 public:
  capture_output_plugin(config_file& cf, std::unique_ptr<cosmology::calculator>& pcc)
      : output_plugin(cf, pcc, "capture") {
    mkdir(fname_.c_str(), 0777);
    const std::string t = cf.get_value_safe<std::string>("output", "capture_type", "particles");
    auto parse = [](const std::string& v) {
      return v == "field_lagrangian" ? output_type::field_lagrangian
                                     : (v == "field_eulerian" ? output_type::field_eulerian : output_type::particles);
    };
    type_ = parse(t);
    type_baryon_ = parse(cf.get_value_safe<std::string>("output", "capture_type_baryon", t));
    real64_ = cf.get_value_safe<bool>("output", "capture_64bit_reals", true);
    id64_ = cf.get_value_safe<bool>("output", "capture_64bit_ids", true);
    const double L = cf.get_value<double>("setup", "BoxLength");
    lunit_ = cf.get_value_safe<double>("output", "capture_lunit", L);
    vunit_ = cf.get_value_safe<double>("output", "capture_vunit", L);
    munit_ = cf.get_value_safe<double>("output", "capture_munit", 1.0);
    const double astart = 1.0 / (1.0 + cf.get_value<double>("setup", "zstart"));
    std::ofstream o(fname_ + "/scalars.txt");
    o << std::setprecision(17);
    o << "astart " << astart << "\n";
    o << "Dplus " << pcc->get_growth_factor(astart) << "\n";
    o << "vfac " << pcc->get_vfact(astart) << "\n";
    for (const char* k : {"pnorm", "sqrtpnorm", "f_b", "n_s", "h", "Omega_m", "Omega_b", "Omega_r", "Omega_k", "Omega_DE",
                          "H0", "sigma_8", "Tcmb"})
      o << k << " " << pcc->cosmo_param_[k] << "\n";
  }

  void write_particle_data(const particle::container& pc, const cosmo_species& s, double Omega) override {
    const std::string p = fname_ + "/" + species_name(s) + "_";
    const size_t np = pc.get_local_num_particles();
    if (real64_) {
      write_npy(p + "pos.npy", pc.get_pos64_ptr(), 3 * np, "<f8", {np, 3});
      write_npy(p + "vel.npy", pc.get_vel64_ptr(), 3 * np, "<f8", {np, 3});
      if (pc.bhas_individual_masses_) write_npy(p + "mass.npy", pc.get_mass64_ptr(), np, "<f8", {np});
    } else {
      write_npy(p + "pos.npy", pc.get_pos32_ptr(), 3 * np, "<f4", {np, 3});
      write_npy(p + "vel.npy", pc.get_vel32_ptr(), 3 * np, "<f4", {np, 3});
      if (pc.bhas_individual_masses_) write_npy(p + "mass.npy", pc.get_mass32_ptr(), np, "<f4", {np});
    }
    if (id64_) write_npy(p + "ids.npy", pc.get_ids64_ptr(), np, "<u8", {np});
    else write_npy(p + "ids.npy", pc.get_ids32_ptr(), np, "<u4", {np});
    std::ofstream o(p + "omega.txt");
    o << std::setprecision(17) << Omega << "\n";
  }

  void write_grid_data(const Grid_FFT<real_t>& g, const cosmo_species& s, const fluid_component& c) override {
    const size_t n0 = g.size(0), n1 = g.size(1), n2 = g.size(2);
    std::vector<double> v(n0 * n1 * n2);
    for (size_t i = 0; i < n0; ++i)
      for (size_t j = 0; j < n1; ++j)
        for (size_t k = 0; k < n2; ++k) v[(i * n1 + j) * n2 + k] = g.relem(i, j, k);
    write_npy(fname_ + "/" + species_name(s) + "_" + component_name(c) + ".npy", v.data(), v.size(), "<f8",
              {n0, n1, n2});
    if (c == fluid_component::density) {
      // the reference's own power-spectrum estimator on a copy of the field,
      // at full precision (Grid_FFT::Compute_PowerSpectrum, src/grid_fft.cc:1133-1210)
      Grid_FFT<real_t> cp({n0, n1, n2}, {g.length_[0], g.length_[1], g.length_[2]});
      for (size_t i = 0; i < n0; ++i)
        for (size_t j = 0; j < n1; ++j)
          for (size_t k = 0; k < n2; ++k) cp.relem(i, j, k) = g.relem(i, j, k);
      std::vector<double> bk, bp, be;
      std::vector<size_t> bc;
      cp.Compute_PowerSpectrum(bk, bp, be, bc);
      std::vector<double> tab;
      for (size_t b = 0; b < bk.size(); ++b) {
        tab.push_back(bk[b]);
        tab.push_back(bp[b]);
        tab.push_back(be[b]);
        tab.push_back((double)bc[b]);
      }
      write_npy(fname_ + "/" + species_name(s) + "_pk.npy", tab.data(), tab.size(), "<f8", {bk.size(), 4});
    }
  }

  output_type write_species_as(const cosmo_species& s) const override {
    return s == cosmo_species::baryon ? type_baryon_ : type_;
  }
  bool has_64bit_reals() const override { return real64_; }
  bool has_64bit_ids() const override { return id64_; }
  real_t position_unit() const override { return lunit_; }
  real_t velocity_unit() const override { return vunit_; }
  real_t mass_unit() const override { return munit_; }
};

output_plugin_creator_concrete<capture_output_plugin> creator_capture("capture");

}  // namespace
