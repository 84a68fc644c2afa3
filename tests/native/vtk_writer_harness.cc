// Host harness of the drop-in driver's VTK writer (no GPU).
//
//   vtk_writer_harness selftest
//     Formats ~3M doubles (random bit patterns over the whole exponent
//     range, mesh coordinates, decimal fractions, zeros, infinities, NaNs)
//     with the writer's fast formatter and with std::ostream's default
//     formatting, which the reference's PvdFileWriter2D uses; prints the
//     mismatch count.
//
//   vtk_writer_harness series <base> <module> <nx> <ny> <dx> <dy> [--particles]
//     Reads output calls from stdin, one per line:
//       dump <call> <time> <ncell> {<name> <file>}... <nnode> {<name> <file>}...
//     (<file>: raw little-endian doubles; numbers in any strtod form, hex
//     floats keep doubles exact) and writes them as the driver does.
#include <cinttypes>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <memory>
#include <random>
#include <sstream>
#include <string>
#include <vector>

#include "pvd_writer.h"

namespace {

std::string via_ostream(double x) {
  std::ostringstream os;
  os << x;
  return os.str();
}

int selftest() {
  std::mt19937_64 rng(12345);
  std::vector<double> xs = {0.0, -0.0, 1.0, -1.0, 0.1, 1e-300, 4.9e-324, -4.9e-324,
                            2.2250738585072014e-308, 1.7976931348623157e308,
                            HUGE_VAL, -HUGE_VAL, std::nan(""), -std::nan(""),
                            999999.5, 999999.4999999, 9.999995, 0.000099999949,
                            1e-5, 1e-4, 123456789.0, 1e16, 0.5, 2.5e-7};
  for (int i = 0; i < 2000000; ++i) {
    uint64_t b = rng();
    double x;
    std::memcpy(&x, &b, sizeof x);
    xs.push_back(x);
  }
  std::uniform_real_distribution<double> u(-2.0, 2.0);
  for (int i = 0; i < 1000000; ++i) xs.push_back(u(rng) * std::pow(10.0, (int)(rng() % 40) - 20));
  for (int i = 0; i < 4097; ++i) {
    xs.push_back(0.005 * (double)(size_t)i);
    xs.push_back((7.0 / 1792) * (double)(size_t)i);
    xs.push_back(i * 1e-3);
    xs.push_back(1.0 / (i + 1));
  }
  long bad = 0;
  for (double x : xs) {
    std::string a;
    hydro_out::append_g6(a, x);
    const std::string b = via_ostream(x);
    if (a != b && bad++ < 10)
      std::printf("mismatch: %a fast '%s' ostream '%s'\n", x, a.c_str(), b.c_str());
  }
  std::printf("%zu values, %ld mismatches\n", xs.size(), bad);
  return bad ? 1 : 0;
}

hydro_out::Array load(const std::string& path) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) {
    std::fprintf(stderr, "cannot open %s\n", path.c_str());
    std::exit(2);
  }
  auto v = std::make_shared<std::vector<double>>();
  double buf[4096];
  size_t n;
  while ((n = std::fread(buf, sizeof(double), 4096, f)) > 0) v->insert(v->end(), buf, buf + n);
  std::fclose(f);
  return v;
}

int series(int argc, char** argv) {
  if (argc < 8) return 2;
  hydro_out::Mesh mesh;
  mesh.nx = std::atol(argv[4]);
  mesh.ny = std::atol(argv[5]);
  mesh.dx = std::strtod(argv[6], nullptr);
  mesh.dy = std::strtod(argv[7], nullptr);
  const bool particles = argc > 8 && !std::strcmp(argv[8], "--particles");
  hydro_out::Writer w;
  hydro_out::PvdSeries s(w, argv[3], argv[2], &mesh);
  std::unique_ptr<hydro_out::PvdSeries> p;
  if (particles) p = std::make_unique<hydro_out::PvdSeries>(w, "Particules", argv[2], nullptr);
  const hydro_out::Vars empty_points = {
      {"VolumePart", nullptr}, {"VxPart", nullptr}, {"VyPart", nullptr}};
  std::string line;
  while (std::getline(std::cin, line)) {
    std::istringstream is(line);
    std::string kw, ts;
    int call;
    if (!(is >> kw >> call >> ts) || kw != "dump") continue;
    const double t = std::strtod(ts.c_str(), nullptr);
    hydro_out::Vars cells, nodes;
    int nc = 0, nn = 0;
    is >> nc;
    for (int k = 0; k < nc; ++k) {
      std::string name, file;
      is >> name >> file;
      cells[name] = load(file);
    }
    is >> nn;
    for (int k = 0; k < nn; ++k) {
      std::string name, file;
      is >> name >> file;
      nodes[name] = load(file);
    }
    s.write(call, t, cells, nodes);
    if (p) p->write(call, t, cells, empty_points);
  }
  w.flush();
  const std::string e = w.error();
  if (!e.empty()) {
    std::fprintf(stderr, "%s\n", e.c_str());
    return 3;
  }
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc >= 2 && !std::strcmp(argv[1], "selftest")) return selftest();
  if (argc >= 2 && !std::strcmp(argv[1], "series")) return series(argc, argv);
  std::fprintf(stderr, "usage: vtk_writer_harness selftest | series ...\n");
  return 2;
}
