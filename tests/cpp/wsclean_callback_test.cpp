// Drives AddInversionDataWithCorrectionCallback of the C++ drop-in built as
// WSClean builds it (WGPU_WITH_WSCLEAN), against the stand-in declarations in
// tests/cpp/wsclean_iface: the callback reads the gridder's cached solutions
// through VisibilityModifier and grids on the GPU.  Writes the images of
// four cases and which of the unsupported cases threw.
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <utility>
#include <vector>

#include "wgpu_gridder.h"

template <typename T>
static std::vector<T> read_file(const char *path, size_t n) {
  std::vector<T> v(n);
  FILE *f = std::fopen(path, "rb");
  if (!f || std::fread(v.data(), sizeof(T), n, f) != n) {
    std::fprintf(stderr, "cannot read %s\n", path);
    std::exit(2);
  }
  std::fclose(f);
  return v;
}

template <typename T>
static void write_file(const std::string &path, const std::vector<T> &v) {
  FILE *f = std::fopen(path.c_str(), "wb");
  std::fwrite(v.data(), sizeof(T), v.size(), f);
  std::fclose(f);
}

int main(int argc, char **argv) {
  using namespace wsclean;
  if (argc != 13) {
    std::fprintf(stderr, "usage: W n_rows n_chan n_ant n_times dl uvw freq vis4 ant tof sol "
                         "(prefix from env OUT)\n");
    return 2;
  }
  const size_t W = std::atoi(argv[1]), n_rows = std::atoi(argv[2]), n_chan = std::atoi(argv[3]);
  const size_t n_ant = std::atoi(argv[4]), n_times = std::atoi(argv[5]);
  const double dl = std::atof(argv[6]);
  auto uvw = read_file<double>(argv[7], 3 * n_rows);
  auto freq = read_file<double>(argv[8], n_chan);
  auto vis = read_file<std::complex<float>>(argv[9], n_rows * n_chan * 4);
  auto ant = read_file<std::pair<size_t, size_t>>(argv[10], n_rows);
  auto tof = read_file<size_t>(argv[11], n_rows);
  auto sol = read_file<std::complex<float>>(argv[12], n_times * n_chan * n_ant * 4);
  const std::string prefix = std::getenv("OUT") ? std::getenv("OUT") : "out_";
  const aocommon::BandData band(n_chan);

  auto image = [&](MsGridder &ms, const std::string &name) {
    WGriddingGridder_Simple<float> g(W, W, W, W, dl, dl, 0.0, 0.0, 1, 1e-4);
    g.InitializeInversion();
    g.AddInversionDataWithCorrectionCallback(GainMode::kFull, 4, n_rows, uvw.data(),
                                             freq.data(), n_chan, band, ant.data(), vis.data(),
                                             tof.data(), &ms, n_ant);
    write_file(prefix + name + ".bin", g.RealImage());
  };
  // a facet with full-Jones h5parm solutions: corrections applied
  MsGridder facet;
  facet.SetIsFacet(true);
  facet.original_ms_index_ = 3;
  facet.GetVisibilityModifier().SetSolutions(3, sol, true);
  image(facet, "callback");
  // the same through the explicit solution table
  {
    WGriddingGridder_Simple<float> g(W, W, W, W, dl, dl, 0.0, 0.0, 1, 1e-4);
    GpuCorrectionTable table;
    table.solutions = sol.data();
    table.n_times = n_times;
    table.nparms = 4;
    table.polarization = WGPU_POL_STOKES_I;
    g.InitializeInversion();
    g.AddInversionDataWithCorrections(GainMode::kFull, 4, n_rows, uvw.data(), freq.data(),
                                      n_chan, ant.data(), vis.data(), tof.data(), table, n_ant);
    write_file(prefix + "explicit.bin", g.RealImage());
  }
  // not a facet: no correction, the rows are only collapsed
  MsGridder plain;
  plain.GetVisibilityModifier().SetSolutions(0, sol, true);
  image(plain, "uncorrected");
  // the cases the device path rejects
  std::vector<int> threw;
  MsGridder dd = facet;
  dd.psf_mode_ = PsfMode::kDirectionDependent;
  MsGridder beam = facet;
  beam.settings_.applyFacetBeam = true;
  for (MsGridder *ms : {&dd, &beam}) {
    int t = 0;
    try {
      image(*ms, "rejected");
    } catch (const std::runtime_error &) {
      t = 1;
    }
    threw.push_back(t);
  }
  write_file(prefix + "threw.bin", threw);
  return 0;
}
