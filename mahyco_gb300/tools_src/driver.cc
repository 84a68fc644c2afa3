// mahyco_gb300_run: drop-in command-line driver of the GPU hydro path.
//
//   mahyco_gb300_run <deck> [--output-dir BASE|none] [--device N]
//                    [--format-threads K] [--quiet]
//
// Same command line and same output as the reference executable (main.cc
// :13-62): reads the positional deck, runs the scheme it names, and writes
// <module>.<call>.vtp / <module>.pvd under ./output (BASE/output with
// --output-dir, nothing with "none"), byte-identical to the reference's
// files.  The time loop and its output calls follow Vnr::executeTimeLoopN /
// Vnr::dumpVariables (vnr_remap/VnrRemap.cc:127-287) and
// Eucclhyd::executeTimeLoopN / Eucclhyd::dumpVariables
// (eucclhyd_remap/EucclhydRemap.cc:24-195):
//   * the output call runs at the start of every cycle (file index = call
//     count = cycle number) and writes when t_n >= lastDump + output_time or
//     t_n == 0;
//   * VNR calls it once more after the loop; the loop's last cycle does not
//     swap its state, so that call sees t_n and the pressure, density and
//     energy of the last cycle's start, but the volume fractions and node
//     velocities that the last remap wrote;
//   * Eucclhyd also writes an empty particle file (Particules.*) with each
//     output.
// The GPU runs cycles back to back and stops by itself before a cycle that
// writes (hydro_run_step_to_output); the fields are copied to the host and
// formatted by a thread pool while the GPU continues.
// Exit status: 0 done, 1 bad deck / options or a run aborted by the scheme's
// checks (the reference's exit(1)), 2 a run the GPU path does not take,
// 3 a CUDA or output error.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "hydro_gb300.h"
#include "pvd_writer.h"

namespace {

using hydro_out::Array;
using hydro_out::Vars;

struct Options {
  std::string deck, base;
  int device = 0, threads = 0;
  bool quiet = false;
};

int usage() {
  std::fprintf(stderr,
               "usage: mahyco_gb300_run <deck> [--output-dir BASE|none] [--device N] "
               "[--format-threads K] [--quiet]\n");
  return 1;
}

[[noreturn]] void die(int code, const std::string& what) {
  std::fprintf(stderr, "[ERREUR] %s: %s\n", what.c_str(), hydro_last_error());
  std::exit(code);
}

Array fetch(hydro_run* run, const char* name) {
  const size_t n = hydro_run_field_size(run, name);
  auto v = std::make_shared<std::vector<double>>(n);
  if (!n || hydro_run_fetch(run, name, v->data(), n) != 0) die(3, std::string("fetch ") + name);
  return v;
}

}  // namespace

int main(int argc, char** argv) {
  Options o;
  for (int a = 1; a < argc; ++a) {
    const std::string s = argv[a];
    if (s == "--output-dir" && a + 1 < argc) o.base = argv[++a];
    else if (s == "--device" && a + 1 < argc) o.device = std::atoi(argv[++a]);
    else if (s == "--format-threads" && a + 1 < argc) o.threads = std::atoi(argv[++a]);
    else if (s == "--quiet") o.quiet = true;
    else if (o.deck.empty() && s.rfind("--", 0) != 0) o.deck = s;
    else return usage();
  }
  if (o.deck.empty()) {
    std::fprintf(stderr, "[ERREUR] Fichier de donnees non passé en argument \n");
    return 1;
  }

  hydro_spec spec;
  if (hydro_spec_parse_deck(o.deck.c_str(), &spec) != 0) die(1, "deck " + o.deck);
  hydro_ctx* ctx = nullptr;
  if (hydro_ctx_create(o.device, 0, &ctx) != 0) die(3, "device");
  hydro_run* run = nullptr;
  if (hydro_run_create(ctx, &spec, &run) != 0) die(2, "run");

  const bool vnr = spec.scheme == HYDRO_SCHEME_VNR;
  hydro_out::Mesh mesh;
  mesh.nx = spec.nx;
  mesh.ny = spec.ny;
  mesh.dx = spec.dx;
  mesh.dy = spec.dy;
  hydro_out::Writer writer(o.threads);
  hydro_out::PvdSeries main_series(writer, vnr ? "VnrRemap" : "EucclhydRemap", o.base, &mesh);
  std::unique_ptr<hydro_out::PvdSeries> particles;
  if (!vnr) particles = std::make_unique<hydro_out::PvdSeries>(writer, "Particules", o.base, nullptr);
  const bool out_on = !main_series.disabled();

  // cell variables of the dump; the VNR fraction planes only with several
  // materials and the remap (VnrRemap.cc:269-274)
  std::vector<const char*> cell_names, node_names;
  if (vnr) {
    cell_names = {"Pressure", "Density", "Energy"};
    if (spec.nbmat > 1 && spec.projection == 1) cell_names.push_back("fracvol1");
    if (spec.nbmat > 2 && spec.projection == 1) cell_names.push_back("fracvol2");
    node_names = {"VitesseX", "VitesseY"};
  } else {
    cell_names = {"Pressure", "Density", "F1", "F2", "F3", "VelocityX", "VelocityY", "Energy"};
  }
  Vars last_cells;  // the arrays of the last output (VNR's final call)
  const Vars empty_points = {{"VolumePart", nullptr}, {"VxPart", nullptr}, {"VyPart", nullptr}};

  // without the remap the mesh moves: each output shows the positions of
  // the cycle's start (Vnr::dumpVariables writes m_node_coord_n)
  const bool moving = vnr && spec.projection == 0;
  auto dump = [&](long call, double t, const Vars& cells, const Vars& nodes) {
    main_series.write((int)call, t, cells, nodes,
                      moving ? fetch(run, "node_coord") : hydro_out::Array());
    if (particles) particles->write((int)call, t, cells, empty_points);
    if (!o.quiet) std::printf(" time = %g sortie demandée \n", t);
  };
  auto dump_now = [&](long call, double t) {
    Vars cells, nodes;
    for (const char* n : cell_names) cells[n] = fetch(run, n);
    for (const char* n : node_names) nodes[n] = fetch(run, n);
    last_cells = cells;
    dump(call, t, cells, nodes);
  };

  double last_dump = 0.0, t = 0.0, dt = 0.0, t_start = 0.0;
  long n = 0, n_start = 0;
  int done = 0, paused = 0;
  for (;;) {
    if (hydro_run_time(run, &t, &dt, &n) != 0) die(3, "time");
    // Vnr::dumpVariables / Eucclhyd::dumpVariables at the start of cycle n+1
    if (out_on && (t >= last_dump + spec.output_time || t == 0.)) {
      dump_now(n + 1, t);
      last_dump = t;
    }
    t_start = t;
    n_start = n;
    const double t_out = out_on ? last_dump + spec.output_time : INFINITY;
    if (hydro_run_step_to_output(run, 1 << 20, t_out, &done, &paused) != 0) die(3, "step");
    unsigned err = 0;
    long cell = -1;
    if (hydro_run_error(run, &err, &cell) != 0) die(3, "error word");
    if (err & ~HYDRO_ERR_NEGATIVE) {
      std::fprintf(stderr, "[ERREUR] run aborted by the scheme's checks: code 0x%x at cell %ld\n",
                   err, cell);
      writer.flush();
      return 1;
    }
    if (done) break;
  }
  if (hydro_run_time(run, &t, &dt, &n) != 0) die(3, "time");
  if (vnr && out_on && n == n_start + 1 &&
      (t_start >= last_dump + spec.output_time || t_start == 0.)) {
    // the final call: the last cycle started at t_start, and this output can
    // only be due if that cycle's start wrote one (last_cells)
    Vars cells = last_cells, nodes;
    for (const char* c : {"fracvol1", "fracvol2"})
      if (cells.count(c)) cells[c] = fetch(run, c);
    for (const char* c : node_names) nodes[c] = fetch(run, c);
    dump(n + 1, t_start, cells, nodes);
    last_dump = t_start;
  }
  writer.flush();
  const std::string werr = writer.error();
  hydro_run_destroy(run);
  hydro_ctx_destroy(ctx);
  if (!werr.empty()) {
    std::fprintf(stderr, "[ERREUR] output: %s\n", werr.c_str());
    return 3;
  }
  if (!o.quiet) std::printf("%ld cycles, t = %.8e\n", n, t);
  return 0;
}
