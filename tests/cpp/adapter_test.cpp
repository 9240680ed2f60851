// Drives the C++ drop-in class (include/wgpu_gridder.h) the way WSClean's
// WGriddingMSGridder does: construct, InitializeInversion, AddInversionData
// in chunks, FinalizeImage, RealImage, InitializePrediction,
// PredictVisibilities.  Inputs are read from and outputs written to raw
// binary files given on the command line; the Python test compares them with
// the oracle.
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "wgpu_gridder.h"
#include "wgpu_imageweights.h"

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
  if (argc != 12) {
    std::fprintf(stderr,
                 "usage: adapter_test width width_t n_rows n_chan dl eps uvw freq vis model out_prefix\n");
    return 2;
  }
  const size_t W = std::atoi(argv[1]), Wt = std::atoi(argv[2]);
  const size_t n_rows = std::atoi(argv[3]), n_chan = std::atoi(argv[4]);
  const double dl = std::atof(argv[5]), eps = std::atof(argv[6]);
  auto uvw = read_file<double>(argv[7], 3 * n_rows);
  auto freq = read_file<double>(argv[8], n_chan);
  auto vis = read_file<std::complex<float>>(argv[9], n_rows * n_chan);
  auto model = read_file<float>(argv[10], W * W);
  std::string prefix = argv[11];
  try {
    wsclean::WGriddingGridder_Simple<double> g(W, W, Wt, Wt, dl, dl, 0.0, 0.0, 4, eps);
    wsclean::WGriddingGridderBase &base = g;
    base.InitializeInversion();
    const size_t half = n_rows / 2;
    base.AddInversionData(half, n_chan, uvw.data(), freq.data(), vis.data());
    base.AddInversionData(n_rows - half, n_chan, uvw.data() + 3 * half, freq.data(),
                          vis.data() + half * n_chan);
    base.FinalizeImage(1.0);
    write_file(prefix + "image.bin", base.RealImage());
    // FinishInversion: resampled to (W + 32)^2, trimmed to Wt^2
    write_file(prefix + "finish.bin", g.FinishInversion(W + 32, W + 32, Wt, Wt));
    base.InitializePrediction(model.data());
    std::vector<std::complex<float>> pred(n_rows * n_chan);
    base.PredictVisibilities(n_rows, n_chan, uvw.data(), freq.data(), pred.data());
    write_file(prefix + "pred.bin", pred);
    // Corrected prediction with one diagonal gain g for every antenna, time
    // and channel: the XX mode writes g * V * conj(g) = |g|^2 V.
    const size_t n_ant = 3;
    std::vector<std::pair<size_t, size_t>> antennas(n_rows);
    std::vector<size_t> time_offsets(n_rows, 0);
    for (size_t r = 0; r < n_rows; ++r) antennas[r] = {r % n_ant, (r + 1) % n_ant};
    std::vector<std::complex<float>> solutions(n_chan * n_ant * 2,
                                               std::complex<float>(1.5f, 0.5f));
    wsclean::GpuCorrectionTable table;
    table.solutions = solutions.data();
    table.n_times = 1;
    table.nparms = 2;
    std::vector<std::complex<float>> pred_corr(n_rows * n_chan);
    g.PredictVisibilitiesWithCorrections(wsclean::GainMode::kXX, 1, n_rows, uvw.data(),
                                         freq.data(), n_chan, antennas.data(),
                                         time_offsets.data(), table, n_ant,
                                         pred_corr.data());
    write_file(prefix + "pred_corr.bin", pred_corr);
    // raw rows with uniform imaging weights (unit visibility weights)
    {
      std::vector<float> ones(n_rows * n_chan, 1.0f);
      wsclean::GpuImageWeights iw(WGPU_WEIGHT_UNIFORM, 0.0, Wt, Wt, dl, dl, false, 1.0);
      iw.Grid(n_rows, n_chan, 1, uvw.data(), freq.data(), ones.data());
      iw.FinishGridding();
      wsclean::WGriddingGridder_Simple<double> g2(W, W, Wt, Wt, dl, dl, 0.0, 0.0, 1, eps);
      wgpu_row_weighting_t rw = {WGPU_PSF_NONE, 0.0, 0.0, 0, WGPU_VISW_NORMAL, WGPU_POL_STOKES_I};
      wgpu_weight_sums_t sums = {0.0, 0.0, 0.0, 0};
      g2.InitializeInversion();
      g2.AddInversionRows(iw.handle(), rw, 1, n_rows, n_chan, uvw.data(), freq.data(),
                          vis.data(), ones.data(), nullptr, nullptr, sums);
      g2.FinalizeImage(1.0);
      write_file(prefix + "rows.bin", g2.RealImage());
      std::vector<double> s4 = {sums.visibility_weight_sum, sums.max_gridded_weight,
                                sums.total_weight, (double)sums.gridded_visibility_count};
      write_file(prefix + "sums.bin", s4);
    }
    // bad argument -> std::runtime_error, as the reference's MR_assert throws
    bool threw = false;
    try {
      wsclean::WGriddingGridder_Simple<float> bad(W, W, Wt, Wt, dl, dl, 0.0, 0.0, 1, eps, 3);
    } catch (const std::runtime_error &) {
      threw = true;
    }
    if (!threw) {
      std::fprintf(stderr, "verbosity 3 was accepted\n");
      return 1;
    }
  } catch (const std::exception &e) {
    std::fprintf(stderr, "%s\n", e.what());
    return 1;
  }
  std::printf("adapter ok\n");
  return 0;
}
