// Drives libm2cg through the C++ adapter (include/m2cg.hpp) the way a
// reference-shaped driver would: configuration and state from files written
// by the test, then ComputeTimeStepSize, ComputeResidual, one
// ComputeRiemannSolution and one ComputeNumericalFluxAtCellInterface, n steps,
// and the results back to files.  Exit codes: 0 ok, 2 bad usage or input,
// 3 the library raised (message on stdout; "no CUDA device" without a GPU).
#include <cstdio>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "m2cg.hpp"

template <class T>
static bool read_file(const std::string& path, std::vector<T>& v, size_t n) {
  std::ifstream f(path, std::ios::binary);
  v.resize(n);
  return (bool)f.read(reinterpret_cast<char*>(v.data()), (std::streamsize)(n * sizeof(T)));
}

template <class T>
static void write_file(const std::string& path, const T* p, size_t n) {
  std::ofstream f(path, std::ios::binary);
  f.write(reinterpret_cast<const char*>(p), (std::streamsize)(n * sizeof(T)));
}

int main(int argc, char** argv) {
  if (argc != 4) {
    std::printf("usage: adapter_check <input prefix> <steps> <output prefix>\n");
    return 2;
  }
  const std::string in = argv[1], out = argv[3];
  const int steps = std::stoi(argv[2]);
  std::vector<char> raw;
  if (!read_file(in + "cfg.bin", raw, sizeof(m2cg_config))) return 2;
  m2cg_config cfg;
  std::memcpy(&cfg, raw.data(), sizeof(cfg));
  const size_t n = (size_t)cfg.nx * cfg.ny * cfg.nz;
  std::vector<double> V, Phi;
  std::vector<int32_t> ID;
  if (!read_file(in + "V.bin", V, 5 * n) || !read_file(in + "ID.bin", ID, n) || !read_file(in + "phi.bin", Phi, n))
    return 2;
  try {
    m2cg::Solver s(cfg);
    s.Upload(V.data(), ID.data(), Phi.data());
    double dtcfl[2];
    s.ComputeTimeStepSize(dtcfl[0], dtcfl[1]);
    std::vector<double> R(5 * n);
    s.ComputeResidual(R.data());
    // the first interface face along x between the first two cells of different ID
    double rs[16] = {0};
    for (size_t c = 0; c + 1 < n; c++) {
      if (ID[c] != ID[c + 1] && (c + 1) % cfg.nx != 0) {
        const double dir[3] = {1.0, 0.0, 0.0};
        int id = -1;
        rs[15] = s.ComputeRiemannSolution(dir, &V[5 * c], ID[c], &V[5 * (c + 1)], ID[c + 1], rs, id, rs + 5, rs + 10);
        rs[15] += 10.0 * id;
        break;
      }
    }
    double F[5];
    s.ComputeNumericalFluxAtCellInterface(0, &V[0], &V[5], ID[0], F);
    m2cg_counters c = s.Run(steps);
    s.Download(V.data(), ID.data(), Phi.data());
    write_file(out + "dt.bin", dtcfl, 2);
    write_file(out + "R.bin", R.data(), R.size());
    write_file(out + "riemann.bin", rs, 16);
    write_file(out + "flux.bin", F, 5);
    write_file(out + "V.bin", V.data(), V.size());
    write_file(out + "ID.bin", ID.data(), ID.size());
    write_file(out + "phi.bin", Phi.data(), Phi.size());
    write_file(out + "counters.bin", &c, 1);
  } catch (const m2cg::Error& e) {
    std::printf("error %d %s\n", (int)e.status, e.what());
    return 3;
  }
  std::printf("ok\n");
  return 0;
}
