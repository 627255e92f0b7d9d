// The project RNG plugin, registered into the reference's own plugin map
// (RNG_plugin_creator_concrete, include/random_plugin.hh:51-65) so that the
// unmodified reference draws the same white noise as the GPU pipeline.  Test
// infrastructure for oracle/_ref.
//
//   [random] generator = PROJECT_PHILOX, seed = <u64>
//       cell c = (i n + j) n + k takes draw c of the project generator
//       (Philox4x32-10 pairs + Box-Muller from IEEE basic operations,
//       monofonic_gb300/csrc/mf_noise.h -- the host side of the plugin whose
//       device twin the pipeline uses);
//   [random] generator = PROJECT_FILE, noise_file = <path>
//       n^3 float64 values, C order, read as the real-space field.
#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

#include <general.hh>
#include <random_plugin.hh>

#include "mf_noise.h"

namespace {

class RNG_project_philox : public RNG_plugin {
  uint64_t seed_;

 public:
  explicit RNG_project_philox(config_file& cf) : RNG_plugin(cf) {
    seed_ = std::stoull(cf.get_value_safe<std::string>("random", "seed", "12345"));
  }
  bool isMultiscale() const override { return false; }
  void Fill_Grid(Grid_FFT<real_t>& g) override {
    const size_t n0 = g.size(0), n1 = g.size(1), n2 = g.size(2);
    const uint64_t ncell = (uint64_t)n0 * n1 * n2;
#pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < (int64_t)((ncell + 1) / 2); ++p) {
      double z[2];
      mf::noise::normal_pair((uint64_t)p, seed_, &z[0], &z[1]);
      for (int h = 0; h < 2; ++h) {
        const uint64_t c = 2 * (uint64_t)p + h;
        if (c >= ncell) break;
        const size_t i = c / (n1 * n2), j = (c / n2) % n1, k = c % n2;
        g.relem(i, j, k) = z[h];
      }
    }
  }
};

class RNG_project_file : public RNG_plugin {
  std::string path_;

 public:
  explicit RNG_project_file(config_file& cf) : RNG_plugin(cf) {
    path_ = cf.get_value<std::string>("random", "noise_file");
  }
  bool isMultiscale() const override { return false; }
  void Fill_Grid(Grid_FFT<real_t>& g) override {
    const size_t n0 = g.size(0), n1 = g.size(1), n2 = g.size(2);
    std::vector<double> v(n0 * n1 * n2);
    FILE* f = std::fopen(path_.c_str(), "rb");
    if (!f) throw std::runtime_error("PROJECT_FILE: cannot open " + path_);
    const size_t got = std::fread(v.data(), sizeof(double), v.size(), f);
    std::fclose(f);
    if (got != v.size()) throw std::runtime_error("PROJECT_FILE: short read from " + path_);
    for (size_t i = 0; i < n0; ++i)
      for (size_t j = 0; j < n1; ++j)
        for (size_t k = 0; k < n2; ++k) g.relem(i, j, k) = v[(i * n1 + j) * n2 + k];
  }
};

RNG_plugin_creator_concrete<RNG_project_philox> creator_philox("PROJECT_PHILOX");
RNG_plugin_creator_concrete<RNG_project_file> creator_file("PROJECT_FILE");

}  // namespace
