// Option defaults and the positional input deck of MaHyCo.
//
// hydro_spec_default mirrors the default member values of the reference's
// option structs (includes/Options.h:9-21, GestionTemps.h:9-18,
// Limiteurs.h:10-25, Eos.h:10-17, CstMesh.h:8-15).
//
// hydro_spec_parse_deck reads a deck with the same sequence of stream
// operations as LectureDonneesClass::LectureDonnees
// (lecture_donnees/LectureDonnees.cc:12-226): one comment line, one value,
// ignore the newline, in a fixed order, with the conditional PenteBorne and
// VNR keys.  Keeping the operations identical keeps the reference's quirks:
// an absent trailing key re-reads the previous word, and an unknown word maps
// to 0 (std::unordered_map::operator[]).
#include <cstdio>
#include <fstream>
#include <string>
#include <unordered_map>

#include "hydro_gb300.h"
#include "internal.h"

namespace {

// Word tables of lecture_donnees/LectureDonnees.h:23-95.
std::unordered_map<std::string, int> casetest_ids() {
  return {{"UnitTestCase", 0},   {"SedovTestCase", 1},   {"TriplePoint", 2},
          {"SodCaseX", 4},       {"SodCaseY", 5},        {"NohTestCase", 6},
          {"AdvectionX", 7},     {"AdvectionY", 8},      {"AdvectionVitX", 9},
          {"AdvectionVitY", 10}, {"BiUnitTestCase", 11}, {"BiSedovTestCase", 12},
          {"BiTriplePoint", 13}, {"BiShockBubble", 14},  {"BiSodCaseX", 15},
          {"BiSodCaseY", 16},    {"BiNohTestCase", 17},  {"BiAdvectionX", 18},
          {"BiAdvectionY", 19},  {"BiAdvectionVitX", 20}, {"BiAdvectionVitY", 21}};
}

}  // namespace

extern "C" int hydro_spec_default(hydro_spec* s) {
  if (!s) return hydro::fail(-1, "hydro_spec_default: null spec");
  *s = hydro_spec{};
  s->scheme = -1;
  s->test_case = -1;
  s->nx = 30;
  s->ny = 30;
  s->dx = 1.2 / 30;
  s->dy = 1.2 / 30;
  s->nbmat = -1;
  for (int m = 0; m < 3; ++m) {
    s->eos[m] = HYDRO_EOS_PERFECT_GAS;
    s->gamma[m] = 1.4;
  }
  s->gamma_scalar = 1.4;
  s->final_time = 1.0;
  s->output_time = 1.0;
  s->dt_init = 0.;
  s->dt_min = 1.0E-10;
  s->cfl = 0.45;
  s->max_cycles = 0;
  s->space_order = 2;
  s->projection = 1;
  s->projection_conservative = 0;
  s->projection_order = 2;
  s->threshold = 1.0E-16;
  s->limiter = -1;
  s->pb = 0;
  s->pb_mixte = 0;
  s->limiter_pure = -1;
  s->pb_complet = 0;
  s->pseudo_centree = 1;
  s->dual_mass_flux = 0;
  s->sans_lagrange = 0;
  s->init_variant = 0;
  s->energy_limit = 5.0;
  return 0;
}

extern "C" int hydro_spec_parse_deck(const char* path, hydro_spec* s) {
  if (!path || !s) return hydro::fail(-1, "hydro_spec_parse_deck: null argument");
  hydro_spec_default(s);
  std::ifstream in(path);
  if (!in) return hydro::fail(-2, std::string("cannot open deck ") + path);

  auto castest = casetest_ids();
  std::unordered_map<std::string, int> schema{
      {"Eucclhyd", 2000}, {"VNR", 2001}, {"CSTS", 2002}, {"MYR", 2003}};
  std::unordered_map<std::string, int> limiteur{
      {"minmod", 300},      {"superBee", 301},  {"vanLeer", 302},
      {"minmodG", 1300},    {"superBeeG", 1301}, {"vanLeerG", 1302},
      {"arithmeticG", 1303}, {"ultrabeeG", 1304}};
  std::unordered_map<std::string, int> ouinon{{"non", 0}, {"oui", 1}};
  std::unordered_map<std::string, int> dual{{"A1", 0}, {"A2", 1}, {"PB", 2}};
  std::unordered_map<std::string, int> eosw{{"Void", 100},
                                            {"PerfectGas", 101},
                                            {"StiffenedGas", 102},
                                            {"Murnhagan", 103},
                                            {"SolidLinear", 104}};
  std::string line, mot;
  int entier = 0;

  std::getline(in, line);
  in >> mot;
  s->test_case = castest[mot];
  in.ignore();
  s->nbmat = (s->test_case < 11) ? 1 : 2;
  if (s->test_case == 13) s->nbmat = 3;
  const int t = s->test_case;
  if (t == 7 || t == 8 || t == 18 || t == 19 || t == 9 || t == 10 || t == 20 ||
      t == 21)
    s->sans_lagrange = 1;

  std::getline(in, line);
  in >> entier;
  s->nx = entier;
  in.ignore();
  std::getline(in, line);
  in >> s->ny;
  in.ignore();
  std::getline(in, line);
  in >> s->dx;
  in.ignore();
  std::getline(in, line);
  in >> s->dy;
  in.ignore();
  std::getline(in, line);
  in >> s->final_time;
  in.ignore();
  std::getline(in, line);
  in >> s->output_time;
  in.ignore();
  std::getline(in, line);
  in >> s->dt_init;
  in.ignore();
  std::getline(in, line);
  in >> s->dt_min;
  in.ignore();
  for (int m = 0; m < s->nbmat; ++m) {
    std::getline(in, line);
    in >> mot;
    s->eos[m] = eosw[mot];
    in.ignore();
  }
  std::getline(in, line);
  in >> mot;
  s->scheme = schema[mot];
  in.ignore();
  std::getline(in, line);
  in >> s->space_order;
  in.ignore();
  std::getline(in, line);
  in >> mot;
  s->projection = ouinon[mot];
  in.ignore();
  std::getline(in, line);
  in >> mot;
  s->projection_conservative = ouinon[mot];
  in.ignore();
  std::getline(in, line);
  in >> s->threshold;
  in.ignore();
  std::getline(in, line);
  in >> s->projection_order;
  in.ignore();
  std::getline(in, line);
  in >> mot;
  s->limiter = limiteur[mot];
  if (s->limiter == -1 || s->limiter == 0)
    return hydro::fail(-3, "deck: limiter '" + mot + "' not supported");
  in.ignore();
  std::getline(in, line);
  in >> mot;
  s->pb = ouinon[mot];
  in.ignore();
  if (s->pb == 1) {
    std::getline(in, line);
    in >> mot;
    s->pb_mixte = ouinon[mot];
    in.ignore();
    std::getline(in, line);
    in >> mot;
    s->limiter_pure = limiteur[mot];
    in.ignore();
    std::getline(in, line);
    in >> mot;
    s->pb_complet = ouinon[mot];
    in.ignore();
  }
  if (s->scheme == HYDRO_SCHEME_VNR) {
    std::getline(in, line);
    in >> mot;
    s->pseudo_centree = ouinon[mot];
    in.ignore();
    if (s->projection == 1) {
      std::getline(in, line);
      in >> mot;
      s->dual_mass_flux = dual[mot];
      in.ignore();
    }
  }
  return 0;
}
