// Oracle harness: drives the UNMODIFIED MaHyCo reference sources (compiled
// from their own directory against oracle/kokkos_shim) and dumps the final
// state at full FP64 precision.  Test infrastructure only: it generates the
// golden vectors under tests/golden/ and checks the C restatement in
// oracle/port/.  Nothing in the product links or runs it.
//
// It mirrors the reference entry point main.cc:13-76 (deck parse, mesh
// generation, scheme construction) and the scheme set-up sequences
// vnr_remap/VnrRemap.cc:330-342 and eucclhyd_remap/EucclhydRemap.cc:273-287,
// then runs the scheme's own executeTimeLoopN().  The sources are compiled
// with class access opened so this file can call the set-up steps one by one and
// read the state afterwards (oracle/ref_fastpath.h); no arithmetic of the
// reference is touched.
//
// usage: mahyco_dump DECK OUTDIR [--cycles N] [--vtk DIR] [--ext-mixed-row]
//                    [--gamma g0,g1,g2] [--cfl C] [--init-only]
//   --cycles N       stop after N cycles (GestTemps::max_time_iterations=N+1,
//                    the loop test at VnrRemap.cc:194-195)
//   --vtk DIR        let the reference write its own VTK output under DIR
//   --gamma ...      per-material gamma (Eos::gammap, includes/Eos.h:16)
//   --cfl C          GestTemps::cfl (read by Eucclhyd only)
//   --ext-mixed-row  bi-material Sod: make the first cell row/column past
//                    the interface a 50/50 mixed cell (extension used by the
//                    2048^2 bi-material workload; same rule as the GPU build)
//   --init-only      dump the state the time loop would start from (after
//                    setUpTimeLoopN) instead of running it: pins the initial
//                    state of cases whose first cycle stops the reference
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "Eucclhyd.h"
#include "Vnr.h"
#include "lecture_donnees/LectureDonnees.h"
#include "mesh/CartesianMesh2D.h"
#include "mesh/CartesianMesh2DGenerator.h"

using namespace nablalib;

namespace {

struct Args {
  std::string deck, outdir, vtk = "none";
  long cycles = -1;
  bool mixed_row = false;
  std::vector<double> gamma;
  double cfl = -1.0;
  bool init_only = false;
};

void dump_raw(const std::string& dir, const std::string& name,
              const double* p, size_t n) {
  std::string path = dir + "/" + name + ".f64";
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) {
    std::perror(path.c_str());
    std::exit(2);
  }
  std::fwrite(p, sizeof(double), n, f);
  std::fclose(f);
}

template <class View>
void dump_scalar(const std::string& dir, const std::string& name,
                 const View& v, size_t n) {
  dump_raw(dir, name, v.data(), n);
}

// Views of RealArray1D<K> are contiguous arrays of K doubles per item.
template <class View>
void dump_vec(const std::string& dir, const std::string& name, const View& v,
              size_t n, size_t k) {
  dump_raw(dir, name, reinterpret_cast<const double*>(v.data()), n * k);
}

// Bi-material Sod extension: the first row (Y case) or column (X case) whose
// cell centre lies past 0.5 becomes a 50/50 mixed cell carrying both states.
template <class S>
void apply_mixed_row(S* s, castestlib::CasTest::Test* test,
                     variableslagremaplib::VariablesLagRemap* varlp, int nx,
                     int ny, double gamma) {
  const bool ycase = (test->Nom == test->BiSodCaseY);
  if (!ycase && test->Nom != test->BiSodCaseX) return;
  const int nline = ycase ? ny : nx;
  int first = -1;
  for (int k = 0; k < nline && first < 0; ++k) {
    size_t c = ycase ? (size_t)k * nx : (size_t)k;
    double r = ycase ? s->m_cell_coord_n0(c)[1] : s->m_cell_coord_n0(c)[0];
    if (!(r < 0.5)) first = k;
  }
  if (first < 0) return;
  const int other = ycase ? nx : ny;
  for (int t = 0; t < other; ++t) {
    size_t c = ycase ? (size_t)first * nx + t : (size_t)t * nx + first;
    const double f0 = 0.5, f1 = 0.5;
    const double r0 = 1.0, r1 = 0.125, p0 = 1.0, p1 = 0.1;
    const double m0 = f0 * r0, m1 = f1 * r1;
    s->m_fracvol_env(c)[0] = f0;
    s->m_fracvol_env(c)[1] = f1;
    s->m_mass_fraction_env(c)[0] = m0 / (m0 + m1);
    s->m_mass_fraction_env(c)[1] = m1 / (m0 + m1);
    s->m_density_env_n0(c)[0] = r0;
    s->m_density_env_n0(c)[1] = r1;
    s->m_pressure_env_n0(c)[0] = p0;
    s->m_pressure_env_n0(c)[1] = p1;
    s->m_density_n0(c) = f0 * r0 + f1 * r1;
    s->m_pressure_n0(c) = f0 * p0 + f1 * p1;
    // same sound-speed rule as the reference init (vnr_remap/Init.cc:172-178)
    s->m_speed_velocity_env_n0(c)[0] = std::sqrt(gamma * r0 / p0);
    s->m_speed_velocity_env_n0(c)[1] = std::sqrt(gamma * r1 / p1);
    s->m_speed_velocity_n0(c) = std::min(s->m_speed_velocity_env_n0(c)[0],
                                         s->m_speed_velocity_env_n0(c)[1]);
    s->m_fracvol_env1(c) = f0;
    s->m_fracvol_env2(c) = f1;
    varlp->mixte(c) = 1;
    varlp->pure(c) = -1;
  }
}

void usage() {
  std::fprintf(stderr,
               "usage: mahyco_dump DECK OUTDIR [--cycles N] [--vtk DIR] "
               "[--gamma a,b,c] [--cfl C] [--ext-mixed-row]\n");
  std::exit(2);
}

Args parse(int argc, char** argv) {
  Args a;
  if (argc < 3) usage();
  a.deck = argv[1];
  a.outdir = argv[2];
  for (int i = 3; i < argc; ++i) {
    std::string k = argv[i];
    if (k == "--cycles" && i + 1 < argc) {
      a.cycles = std::atol(argv[++i]);
    } else if (k == "--vtk" && i + 1 < argc) {
      a.vtk = argv[++i];
    } else if (k == "--init-only") {
      a.init_only = true;
    } else if (k == "--ext-mixed-row") {
      a.mixed_row = true;
    } else if (k == "--cfl" && i + 1 < argc) {
      a.cfl = std::atof(argv[++i]);
    } else if (k == "--gamma" && i + 1 < argc) {
      std::string s = argv[++i];
      size_t pos = 0;
      while (pos <= s.size()) {
        size_t q = s.find(',', pos);
        if (q == std::string::npos) q = s.size();
        a.gamma.push_back(std::atof(s.substr(pos, q - pos).c_str()));
        pos = q + 1;
      }
    } else {
      usage();
    }
  }
  return a;
}

void write_meta(const std::string& dir, const char* scheme, int nx, int ny,
                int nbmat, long cycles, double t, double dt) {
  std::string path = dir + "/meta.txt";
  FILE* f = std::fopen(path.c_str(), "w");
  std::fprintf(f, "scheme %s\nnx %d\nny %d\nnbmat %d\ncycles %ld\n", scheme,
               nx, ny, nbmat, cycles);
  std::fprintf(f, "t %.17g\ndt %.17g\n", t, dt);
  std::fclose(f);
}

}  // namespace

int main(int argc, char** argv) {
  Args a = parse(argc, argv);
  Kokkos::initialize(argc, argv);
  auto scheme = new schemalagrangelib::SchemaLagrangeClass::SchemaLagrange();
  auto o = new optionschemalib::OptionsSchema::Options();
  auto cl = new conditionslimiteslib::ConditionsLimites::Cdl();
  auto lim = new limiteurslib::LimiteursClass::Limiteurs();
  auto eos = new eoslib::EquationDetat::Eos();
  auto test = new castestlib::CasTest::Test();
  auto cstmesh = new cstmeshlib::ConstantesMaillagesClass::ConstantesMaillages();
  auto gt = new gesttempslib::GestionTempsClass::GestTemps();
  LectureDonneesClass lecture;
  lecture.LectureDonnees(a.deck, scheme, o, cstmesh, gt, lim, eos, test);
  if (a.cycles > 0) gt->max_time_iterations = (int)(a.cycles + 1);
  for (size_t i = 0; i < a.gamma.size() && i < 3; ++i) eos->gammap[i] = a.gamma[i];
  if (a.cfl > 0) gt->cfl = a.cfl;

  auto nm = CartesianMesh2DGenerator::generate(
      cstmesh->X_EDGE_ELEMS, cstmesh->Y_EDGE_ELEMS, cstmesh->X_EDGE_LENGTH,
      cstmesh->Y_EDGE_LENGTH);
  const int nx = cstmesh->X_EDGE_ELEMS, ny = cstmesh->Y_EDGE_ELEMS;
  const size_t nc = (size_t)nx * ny, nn = (size_t)(nx + 1) * (ny + 1);
  const std::string& od = a.outdir;

  auto varlp = new variableslagremaplib::VariablesLagRemap(nm);
  auto part = new particleslib::SchemaParticules(nm, cstmesh, gt, test);
  auto proj = new Remap(o, cstmesh, gt, cl, lim, nm, varlp);

  if (scheme->schema == scheme->VNR) {
    auto c = new Vnr(o, cstmesh, gt, test, cl, lim, part, eos, nm, varlp, proj,
                     a.vtk);
    c->initBoundaryConditions();
    c->initCellPos();
    c->init();
    if (a.mixed_row) apply_mixed_row(c, test, varlp, nx, ny, eos->gamma);
    c->initSubVol();
    c->initMeshGeometryForFaces();
    proj->FacesOfNode();
    c->computeCellMass();
    if (o->sansLagrange == 0) c->initDeltaT();
    if (o->sansLagrange == 0) c->initInternalEnergy();
    if (o->sansLagrange == 0) c->initPseudo();
    c->setUpTimeLoopN();
    c->computeNodeMass();
    if (a.init_only) {
      // the state the time loop starts from (after setUpTimeLoopN's copies)
      dump_scalar(od, "density", c->m_density_n, nc);
      dump_scalar(od, "pressure", c->m_pressure_n, nc);
      dump_scalar(od, "energy", c->m_internal_energy_n, nc);
      dump_scalar(od, "sound_speed", c->m_speed_velocity_n, nc);
      dump_scalar(od, "pseudo", c->m_pseudo_viscosity_n, nc);
      dump_scalar(od, "divu", c->m_divu_n, nc);
      dump_scalar(od, "cell_mass", c->m_cell_mass, nc);
      dump_vec(od, "density_env", c->m_density_env_n, nc, 3);
      dump_vec(od, "energy_env", c->m_internal_energy_env_n, nc, 3);
      dump_vec(od, "pressure_env", c->m_pressure_env_n, nc, 3);
      dump_vec(od, "fracvol_env", c->m_fracvol_env, nc, 3);
      dump_vec(od, "mass_fraction_env", c->m_mass_fraction_env, nc, 3);
      dump_vec(od, "node_velocity", c->m_node_velocity_n, nn, 2);
      dump_scalar(od, "node_mass", c->m_node_mass, nn);
      write_meta(od, "VNR", nx, ny, o->nbmat, 0, gt->t_n, gt->deltat_n);
      Kokkos::finalize();
      return 0;
    }
    c->executeTimeLoopN();
    // The last cycle does not swap (VnrRemap.cc:198): final state is _nplus1.
    dump_scalar(od, "density", c->m_density_nplus1, nc);
    dump_scalar(od, "pressure", c->m_pressure_nplus1, nc);
    dump_scalar(od, "energy", c->m_internal_energy_nplus1, nc);
    dump_scalar(od, "sound_speed", c->m_speed_velocity_nplus1, nc);
    dump_scalar(od, "pseudo", c->m_pseudo_viscosity_nplus1, nc);
    dump_scalar(od, "divu", c->m_divu_nplus1, nc);
    dump_scalar(od, "cell_mass", c->m_cell_mass, nc);
    dump_vec(od, "density_env", c->m_density_env_nplus1, nc, 3);
    dump_vec(od, "energy_env", c->m_internal_energy_env_nplus1, nc, 3);
    dump_vec(od, "pressure_env", c->m_pressure_env_nplus1, nc, 3);
    dump_vec(od, "fracvol_env", c->m_fracvol_env, nc, 3);
    dump_vec(od, "mass_fraction_env", c->m_mass_fraction_env, nc, 3);
    dump_vec(od, "node_velocity", c->m_node_velocity_nplus1, nn, 2);
    dump_scalar(od, "node_mass", c->m_node_mass, nn);
    write_meta(od, "VNR", nx, ny, o->nbmat, c->n, gt->t_nplus1,
               gt->deltat_nplus1);
  } else if (scheme->schema == scheme->Eucclhyd) {
    auto c = new Eucclhyd(o, cstmesh, gt, test, cl, lim, part, eos, nm, varlp,
                          proj, a.vtk);
    c->computeCornerNormal();
    c->initMeshGeometryForCells();
    c->initVpAndFpc();
    c->initBoundaryConditions();
    c->initCellInternalEnergy();
    c->initCellVelocity();
    c->initDensity();
    c->initMeshGeometryForFaces();
    c->setUpTimeLoopN();
    if (a.init_only) {
      dump_scalar(od, "density", c->m_density_n, nc);
      dump_scalar(od, "energy", c->m_internal_energy_n, nc);
      dump_vec(od, "cell_velocity", c->m_cell_velocity_n, nc, 2);
      dump_vec(od, "density_env", c->m_density_env_n, nc, 3);
      dump_vec(od, "energy_env", c->m_internal_energy_env_n, nc, 3);
      dump_vec(od, "fracvol_env", c->m_fracvol_env, nc, 3);
      dump_vec(od, "mass_fraction_env", c->m_mass_fraction_env, nc, 3);
      dump_vec(od, "node_velocity", c->m_node_velocity_n, nn, 2);
      write_meta(od, "Eucclhyd", nx, ny, o->nbmat, 0, gt->t_n, gt->deltat_n);
      Kokkos::finalize();
      return 0;
    }
    c->executeTimeLoopN();
    dump_scalar(od, "density", c->m_density_nplus1, nc);
    dump_scalar(od, "pressure", c->m_pressure, nc);
    dump_scalar(od, "energy", c->m_internal_energy_nplus1, nc);
    dump_scalar(od, "sound_speed", c->m_speed_velocity, nc);
    dump_vec(od, "cell_velocity", c->m_cell_velocity_nplus1, nc, 2);
    dump_vec(od, "density_env", c->m_density_env_nplus1, nc, 3);
    dump_vec(od, "energy_env", c->m_internal_energy_env_nplus1, nc, 3);
    dump_vec(od, "fracvol_env", c->m_fracvol_env, nc, 3);
    dump_vec(od, "mass_fraction_env", c->m_mass_fraction_env, nc, 3);
    dump_vec(od, "node_velocity", c->m_node_velocity_nplus1, nn, 2);
    write_meta(od, "Eucclhyd", nx, ny, o->nbmat, c->n, gt->t_nplus1,
               gt->deltat_nplus1);
  } else {
    std::fprintf(stderr, "unsupported scheme %d\n", scheme->schema);
    return 2;
  }
  Kokkos::finalize();
  return 0;
}
