// .pmp tokenizer and materials.
//
// Tokenizer semantics follow input::clean / input::get_next_line (input.cxx:4-62):
// tabs become a space (swallowing the next character, as the reference's replace(i, 2, " ")
// does), runs of spaces collapse, lines are trimmed, '#' starts a comment line, and
// blank lines are skipped.  Material reading follows Material::read (Material.cxx:18-131)
// and ConstantNuclearData::read/check (ConstantNuclearData.cxx:4-177).
#include <cerrno>
#include <climits>
#include <cfloat>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <sys/stat.h>

#include <algorithm>

#include "pg_host.hpp"

namespace pg {

namespace {

std::string clean(std::string s) {
  if (s.empty()) return s;
  size_t i;
  while ((i = s.find('\t')) != std::string::npos) s.replace(i, 2, " ");
  while ((i = s.find("  ")) != std::string::npos) s.erase(i, 1);
  if (s == " ") return std::string();
  size_t a = s.find_first_not_of(' ');
  size_t b = s.find_last_not_of(' ');
  if (a == std::string::npos) return std::string();
  s = s.substr(a, b - a + 1);
  if (!s.empty() && s[0] == '#') return std::string();
  return s;
}

}  // namespace

int Tokens::open(const std::string& path) {
  path_ = path;
  std::ifstream in(path);
  PG_CHECK(!in.is_open(), "unable to open " + path);
  std::string line;
  lines_.clear();
  while (std::getline(in, line)) {
    if (!line.empty() && line.back() == '\r') line.pop_back();
    lines_.push_back(line);
  }
  pos_ = 0;
  return 0;
}

std::vector<std::string> Tokens::next() {
  std::vector<std::string> words;
  while (pos_ < lines_.size()) {
    std::string s = clean(lines_[pos_++]);
    if (s.empty()) continue;
    std::istringstream iss(s);
    std::string w;
    while (std::getline(iss, w, ' ')) words.push_back(w);
    break;
  }
  return words;
}

int to_int(const std::string& s, int lo, int hi, int& out) {
  char* end = nullptr;
  errno = 0;
  long v = std::strtol(s.c_str(), &end, 10);
  PG_CHECK(end == s.c_str() || errno != 0, "wrong int value '" + s + "'");
  PG_CHECK(v < lo || v > hi, "out-of-bounds int value");
  out = (int)v;
  return 0;
}

int to_double(const std::string& s, double lo, double hi, double& out) {
  char* end = nullptr;
  errno = 0;
  double v = std::strtod(s.c_str(), &end);
  PG_CHECK(end == s.c_str(), "wrong double value '" + s + "'");
  PG_CHECK(v < lo || v > hi, "out-of-bounds double value");
  out = v;
  return 0;
}

int to_bool(const std::string& s, bool& out) {
  int v;
  PG_TRY(to_int(s, 0, 1, v), "wrong bool value");
  out = v != 0;
  return 0;
}

int Tokens::read_doubles(std::vector<double>& v, size_t n, double lo, double hi) {
  v.clear();
  v.reserve(n);
  while (v.size() < n) {
    std::vector<std::string> line = next();
    PG_CHECK(line.empty(), "missing data in " + path_);
    for (const auto& w : line) {
      PG_CHECK(v.size() >= n, "out-of-bounds data in " + path_);
      double x;
      PG_TRY(to_double(w, lo, hi, x), "wrong data");
      v.push_back(x);
    }
  }
  return 0;
}

int Tokens::read_ints(std::vector<int>& v, size_t n, int lo, int hi) {
  v.clear();
  v.reserve(n);
  while (v.size() < n) {
    std::vector<std::string> line = next();
    PG_CHECK(line.empty(), "missing data in " + path_);
    for (const auto& w : line) {
      PG_CHECK(v.size() >= n, "out-of-bounds data in " + path_);
      int x;
      PG_TRY(to_int(w, lo, hi, x), "wrong data");
      v.push_back(x);
    }
  }
  return 0;
}

std::string resolve_path(const std::string& path, const std::string& base_dir) {
  struct stat st;
  if (path.empty() || path[0] == '/' || stat(path.c_str(), &st) == 0 || base_dir.empty())
    return path;
  return base_dir + "/" + path;
}

// input::read(BoundaryCondition&, ...) (input.cxx:364-404).  Steady state evaluates each
// parameter function at t = 0 (Function.hxx:34-38: a table returns its first value).
int read_bc(const std::vector<std::string>& line, size_t i, Tokens& tok, BoundaryCondition& bc) {
  PG_CHECK(i >= line.size(), "missing boundary-condition type");
  const std::string& t = line[i++];
  if (t == "vacuum") bc.type = BC_VACUUM;
  else if (t == "reflective") bc.type = BC_REFLECTIVE;
  else if (t == "robin") bc.type = BC_ROBIN;
  else if (t == "dirichlet") bc.type = BC_DIRICHLET;
  else if (t == "adiabatic") bc.type = BC_ADIABATIC;
  else if (t == "convection") bc.type = BC_CONVECTION;
  else PG_CHECK(true, "wrong boundary-condition type");
  int m = (bc.type == BC_ROBIN || bc.type == BC_DIRICHLET) ? 1 : (bc.type == BC_CONVECTION ? 2 : 0);
  bc.values.clear();
  if (m == 0) return 0;
  if (line.size() == i + m && !(line.size() == i + 2 && line[i + 1] == "{")) {
    for (int j = 0; j < m; j++) {
      double x;
      PG_TRY(to_double(line[i + j], -DBL_MAX, DBL_MAX, x), "wrong boundary-condition parameter");
      bc.values.push_back(x);
    }
  } else if (line.size() == i + 2 && line[i + 1] == "{") {
    int n;
    PG_TRY(to_int(line[i], 1, INT_MAX, n), "wrong number of time points");
    std::vector<double> t0, y;
    PG_TRY(tok.read_doubles(t0, n, 0.0, DBL_MAX), "wrong time data");
    for (int j = 0; j < m; j++) {
      PG_TRY(tok.read_doubles(y, n, -DBL_MAX, DBL_MAX), "wrong function data");
      bc.values.push_back(y[0]);
    }
    std::vector<std::string> close = tok.next();
    PG_CHECK(close.empty() || close[0] != "}", "missing closing '}' for function data");
  } else {
    PG_CHECK(true, "wrong number of function arguments");
  }
  return 0;
}

// ----------------------------------------------------------------------------------
// Material
// ----------------------------------------------------------------------------------

int Material::read_file(const std::string& path) {
  Tokens tok;
  PG_TRY(tok.open(path), "unable to open " + path);
  PG_TRY(read(tok), "unable to read the material from " + path);
  return 0;
}

int Material::read(Tokens& tok) {
  while (true) {
    std::vector<std::string> line = tok.next();
    if (line.empty() || line[0] == "}") break;
    const std::string& k = line[0];
    if (k == "nuclear-data") {
      PG_CHECK(line.size() != 2 || line[1] != "{", "missing opening '{' for constant nuclear data");
      PG_TRY(read_nuclear_data(tok), "unable to read the constant nuclear data");
      has_nd = true;
    } else if (k == "nuclear-data-set") {
      // FeedbackNuclearData::read (FeedbackNuclearData.cxx): reference temperatures and one
      // constant data set per temperature
      PG_CHECK(line.size() != 2 || line[1] != "{", "missing opening '{' for feedback nuclear data");
      feedback_sets.clear();
      tref.clear();
      while (true) {
        std::vector<std::string> l2 = tok.next();
        if (l2.empty() || l2[0] == "}") break;
        if (l2[0] == "temperature") {
          PG_CHECK(l2.size() != 2, "wrong number of arguments for keyword 'temperature'");
          int nt = 0;
          PG_TRY(to_int(l2[1], 0, INT_MAX, nt), "wrong number of temperatures");
          PG_TRY(tok.read_doubles(tref, nt, 0.0, DBL_MAX), "wrong temperature data");
        } else if (l2[0] == "nuclear-data") {
          PG_CHECK(l2.size() != 2 || l2[1] != "{", "missing opening '{' for nuclear data");
          Material set;
          PG_TRY(set.read_nuclear_data(tok), "unable to read the nuclear data");
          set.has_nd = true;
          feedback_sets.push_back(set);
        } else {
          PG_CHECK(true, "unrecognized keyword '" + l2[0] + "'");
        }
      }
      PG_CHECK(feedback_sets.empty() || feedback_sets.size() != tref.size(),
               "one nuclear-data set is needed per reference temperature");
      for (size_t k2 = 1; k2 < tref.size(); k2++)
        PG_CHECK(!(tref[k2] > tref[k2 - 1]), "reference temperatures must increase");
      has_nd = true;
    } else if (k == "precursor-data") {
      PG_CHECK(line.size() != 2 || line[1] != "{", "missing opening '{' for precursor data");
      int npg = 0;
      has_pd = true;
      while (true) {
        std::vector<std::string> l2 = tok.next();
        if (l2.empty() || l2[0] == "}") break;
        if (l2[0] == "precursor-groups") {
          PG_TRY(to_int(l2.at(1), 1, INT_MAX, npg), "wrong number of precursor groups");
        } else if (l2[0] == "lambda") {
          PG_TRY(tok.read_doubles(precursor_lambda, npg, 0.0, DBL_MAX), "wrong precursor decay constants");
        } else if (l2[0] == "beta") {
          PG_TRY(tok.read_doubles(precursor_beta, npg, 0.0, DBL_MAX), "wrong precursor fractions");
          beta_total = 0.0;
          for (double b : precursor_beta) beta_total += b;  // PrecursorData.cxx:44-45
        } else {
          PG_CHECK(true, "unrecognized keyword '" + l2[0] + "'");
        }
      }
      num_precursor_groups = npg;
      PG_CHECK(precursor_lambda.size() != (size_t)npg || precursor_beta.size() != (size_t)npg,
               "missing precursor decay constants or fractions");
    } else if (k == "thermal-properties") {
      PG_CHECK(line.size() < 2, "wrong number of arguments for keyword 'thermal-properties'");
    } else if (k == "fuel") {
      PG_TRY(to_bool(line.at(1), fuel), "wrong switch for fuel materials");
    } else if (k == "bc") {
      PG_TRY(to_bool(line.at(1), bc), "wrong switch for boundary-condition materials");
    } else if (k == "split") {
      PG_TRY(to_bool(line.at(1), split), "wrong switch for split materials");
    } else {
      PG_CHECK(true, "unrecognized keyword '" + k + "'");
    }
  }
  if (!feedback_sets.empty()) {
    // FeedbackNuclearData::check(beta_total): every set is completed as constant data is;
    // the material's own arrays hold the first set (the data at the lowest temperature)
    for (auto& set : feedback_sets) {
      set.beta_total = beta_total;
      PG_TRY(set.finish_nuclear_data(), "wrong nuclear data");
      PG_CHECK(set.num_groups != feedback_sets[0].num_groups, "wrong number of energy groups");
    }
    const Material& s0 = feedback_sets[0];
    num_groups = s0.num_groups;
    sigma_t = s0.sigma_t, nu_sigma_f = s0.nu_sigma_f, kappa_sigma_f = s0.kappa_sigma_f, sigma_tr = s0.sigma_tr;
    diffusion = s0.diffusion, chi_prompt = s0.chi_prompt, chi_delayed = s0.chi_delayed, chi = s0.chi;
    velocity = s0.velocity, sigma_s = s0.sigma_s;
  } else if (has_nd) {
    PG_TRY(finish_nuclear_data(), "wrong nuclear data");
  }
  return 0;
}

// FeedbackNuclearData::interpolate and its getters (FeedbackNuclearData.hxx:60-140): below
// the first reference temperature the first set, above the last the last set, otherwise
// the linear interpolation between the two sets around T (lower_bound of T).  A
// temperature equal to the first reference value makes the reference read the set before
// the first one; the first set is used here.
void Material::at(double T, Material& out) const {
  if (feedback_sets.empty()) {
    out = *this;
    return;
  }
  int i1, i2;
  double f;
  if (T < tref.front()) {
    i1 = i2 = 0, f = 0.0;
  } else if (T > tref.back()) {
    i1 = i2 = (int)tref.size() - 1, f = 0.0;
  } else {
    i2 = (int)(std::lower_bound(tref.begin(), tref.end(), T) - tref.begin());
    if (i2 == 0) {
      i1 = 0, f = 0.0;
    } else {
      i1 = i2 - 1;
      f = (T - tref[i1]) / (tref[i2] - tref[i1]);
    }
  }
  const Material& a = feedback_sets[i1];
  const Material& b = feedback_sets[i2];
  auto mix = [&](const std::vector<double>& x, const std::vector<double>& y, std::vector<double>& o) {
    o.resize(x.size());
    for (size_t k = 0; k < x.size() && k < y.size(); k++) o[k] = (1.0 - f) * x[k] + f * y[k];
  };
  out = *this;
  out.feedback_sets.clear();
  out.tref.clear();
  mix(a.sigma_t, b.sigma_t, out.sigma_t);
  mix(a.nu_sigma_f, b.nu_sigma_f, out.nu_sigma_f);
  mix(a.kappa_sigma_f, b.kappa_sigma_f, out.kappa_sigma_f);
  mix(a.sigma_tr, b.sigma_tr, out.sigma_tr);
  mix(a.diffusion, b.diffusion, out.diffusion);
  mix(a.chi_prompt, b.chi_prompt, out.chi_prompt);
  mix(a.chi_delayed, b.chi_delayed, out.chi_delayed);
  mix(a.chi, b.chi, out.chi);
  mix(a.velocity, b.velocity, out.velocity);
  mix(a.sigma_s, b.sigma_s, out.sigma_s);
}

int Material::read_nuclear_data(Tokens& tok) {
  while (true) {
    std::vector<std::string> line = tok.next();
    if (line.empty() || line[0] == "}") break;
    const std::string& k = line[0];
    if (k == "energy-groups") {
      PG_TRY(to_int(line.at(1), 1, INT_MAX, num_groups), "wrong number of energy groups");
      continue;
    }
    PG_CHECK(line.size() != 1, "wrong number of arguments for keyword '" + k + "'");
    PG_CHECK(num_groups < 1, "energy-groups must come first in nuclear data");
    std::vector<double>* dst = nullptr;
    if (k == "sigma-total") dst = &sigma_t;
    else if (k == "nu-sigma-fission") dst = &nu_sigma_f;
    else if (k == "kappa-sigma-fission") dst = &kappa_sigma_f;
    else if (k == "sigma-transport") dst = &sigma_tr;
    else if (k == "diffusion-coefficient") dst = &diffusion;
    else if (k == "fission-spectrum" || k == "fission-spectrum-prompt") dst = &chi_prompt;
    else if (k == "fission-spectrum-delayed") dst = &chi_delayed;
    else if (k == "neutron-velocity") dst = &velocity;
    if (dst) {
      PG_TRY(tok.read_doubles(*dst, num_groups, 0.0, DBL_MAX), "wrong " + k);
    } else if (k == "sigma-scattering") {
      sigma_s.clear();
      for (int g = 0; g < num_groups; g++) {
        std::vector<std::string> row = tok.next();
        PG_CHECK((int)row.size() != num_groups, "wrong scattering cross sections");
        for (const auto& w : row) {
          double x;
          PG_TRY(to_double(w, 0.0, DBL_MAX, x), "wrong scattering cross sections");
          sigma_s.push_back(x);
        }
      }
    } else {
      PG_CHECK(true, "unrecognized keyword '" + k + "'");
    }
  }
  return 0;
}

// ConstantNuclearData::check(beta_total) (ConstantNuclearData.cxx:129-177).
int Material::finish_nuclear_data() {
  const int G = num_groups;
  if (!nu_sigma_f.empty() || !chi_prompt.empty()) {
    PG_CHECK(nu_sigma_f.empty(), "missing nu-fission cross sections");
    PG_CHECK(chi_prompt.empty(), "missing fission spectrum");
  }
  if (nu_sigma_f.empty()) nu_sigma_f.assign(G, 0.0);
  if (kappa_sigma_f.empty()) {
    const double nu = 2.4355, kappa = 3.2e-11;  // ConstantNuclearData.hxx:27
    const double f = kappa / nu;
    kappa_sigma_f = nu_sigma_f;
    for (auto& x : kappa_sigma_f) x *= f;
  }
  if (chi_prompt.empty()) chi_prompt.assign(G, 0.0);
  if (chi_delayed.empty()) chi_delayed = chi_prompt;
  if (beta_total > 0.0) {
    chi.assign(G, 0.0);
    for (int g = 0; g < G; g++) chi[g] = (1.0 - beta_total) * chi_prompt[g] + beta_total * chi_delayed[g];
  } else {
    chi = chi_prompt;
  }
  if (!sigma_tr.empty()) {
    PG_CHECK(!diffusion.empty(),
             "transport cross sections can only be defined if diffusion coefficients are not");
    diffusion.assign(G, 0.0);
    for (int g = 0; g < G; g++) diffusion[g] = 1.0 / (3.0 * sigma_tr[g]);
  }
  return 0;
}

// ConstantNuclearData::check(G, diffusion, transient) (ConstantNuclearData.cxx:180-200).
int Material::check_for_solver(int G, bool diffusion_solver, bool transient) const {
  PG_CHECK(!has_nd, "missing nuclear data");
  for (const auto& set : feedback_sets)  // FeedbackNuclearData::check(G, diffusion, transient)
    PG_TRY(set.check_for_solver(G, diffusion_solver, transient), "wrong nuclear data");
  PG_CHECK(num_groups != G, "wrong number of energy groups");
  PG_CHECK(sigma_t.empty(), "missing total cross sections");
  PG_CHECK(sigma_s.empty(), "missing scattering cross sections");
  PG_CHECK(chi.empty(), "missing effective fission spectrum");
  if (diffusion_solver) PG_CHECK(diffusion.empty(), "missing diffusion coefficients");
  if (transient) {
    PG_CHECK(chi_prompt.empty(), "missing prompt fission spectrum");
    PG_CHECK(chi_delayed.empty(), "missing delayed fission spectrum");
    PG_CHECK(velocity.empty(), "missing neutron velocities");
  }
  return 0;
}

}  // namespace pg
