// namelist.cpp -- minimal Fortran namelist reader for test.nml files.
#include "namelist.h"

#include <algorithm>
#include <cctype>
#include <cstdlib>
#include <fstream>
#include <map>
#include <set>
#include <sstream>

namespace {

std::string lower(std::string s) {
  std::transform(s.begin(), s.end(), s.begin(), [](unsigned char c) { return (char)std::tolower(c); });
  return s;
}

std::string trim(const std::string& s) {
  size_t a = s.find_first_not_of(" \t\r\n,");
  size_t b = s.find_last_not_of(" \t\r\n,");
  return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
}

// Fortran real literal: d/D/q/Q exponent letters mean double.
bool to_double(std::string v, double* out) {
  for (char& c : v)
    if (c == 'd' || c == 'D' || c == 'q' || c == 'Q') c = 'e';
  char* end = nullptr;
  *out = std::strtod(v.c_str(), &end);
  return end && *end == '\0' && !v.empty();
}

bool to_int(const std::string& v, int* out) {
  char* end = nullptr;
  long x = std::strtol(v.c_str(), &end, 10);
  if (!end || *end != '\0' || v.empty()) return false;
  *out = (int)x;
  return true;
}

std::string unquote(std::string v) {
  if (v.size() >= 2 && (v.front() == '\'' || v.front() == '"') && v.back() == v.front())
    return v.substr(1, v.size() - 2);
  return v;
}

}  // namespace

std::string read_namelist(const std::string& path, RunConfig* cfg) {
  std::ifstream in(path);
  if (!in) return "cannot open " + path;
  std::stringstream ss;
  std::string line;
  while (std::getline(in, line)) {  // drop comments
    bool q = false;
    char qc = 0;
    std::string out;
    for (char c : line) {
      if (q) {
        out += c;
        if (c == qc) q = false;
      } else if (c == '\'' || c == '"') {
        q = true;
        qc = c;
        out += c;
      } else if (c == '!') {
        break;
      } else {
        out += c;
      }
    }
    ss << out << '\n';
  }
  const std::string text = ss.str();
  std::map<std::string, std::map<std::string, std::string>> groups;
  size_t pos = 0;
  while ((pos = text.find('&', pos)) != std::string::npos) {
    size_t nend = pos + 1;
    while (nend < text.size() && (std::isalnum((unsigned char)text[nend]) || text[nend] == '_')) ++nend;
    const std::string name = lower(text.substr(pos + 1, nend - pos - 1));
    size_t close = text.find('/', nend);
    if (close == std::string::npos) return "namelist group &" + name + " is not terminated by /";
    std::string body = text.substr(nend, close - nend);
    // split "key = value" pairs separated by commas or newlines
    std::map<std::string, std::string> items;
    size_t k = 0;
    while (k < body.size()) {
      size_t eq = body.find('=', k);
      if (eq == std::string::npos) break;
      std::string key = lower(trim(body.substr(k, eq - k)));
      size_t next = eq + 1;
      // the value runs until the next "ident =" or the end
      size_t scan = next, vend = body.size();
      while (scan < body.size()) {
        size_t e2 = body.find('=', scan);
        if (e2 == std::string::npos) break;
        size_t b = e2;
        while (b > next && std::isspace((unsigned char)body[b - 1])) --b;
        size_t a = b;
        while (a > next && (std::isalnum((unsigned char)body[a - 1]) || body[a - 1] == '_')) --a;
        if (a < b) {
          vend = a;
          break;
        }
        scan = e2 + 1;
      }
      items[key] = trim(body.substr(next, vend - next));
      k = vend;
    }
    groups[name] = items;
    pos = close + 1;
  }
  for (const char* g : {"run", "mesh", "hydro"})
    if (!groups.count(g)) return std::string("namelist group &") + g + " missing from " + path;

  e2d_default_params(&cfg->p);
  static const std::map<std::string, std::set<std::string>> allowed = {
      {"run", {"tend", "nstepmax", "noutput"}},
      {"mesh", {"nx", "ny", "boundary_type_xmin", "boundary_type_xmax", "boundary_type_ymin", "boundary_type_ymax"}},
      {"hydro", {"gamma0", "cfl", "smallr", "smallc", "niter_riemann", "iorder", "slope_type"}},
      {"other", {"implementationversion"}},
      {"gb300", {"riemann_solver", "precision"}},
  };
  for (const auto& g : groups) {
    auto al = allowed.find(g.first);
    if (al == allowed.end()) continue;
    for (const auto& kv : g.second) {
      const std::string& key = kv.first;
      const std::string& val = kv.second;
      if (!al->second.count(key)) return "unknown key " + key + " in namelist group &" + g.first;
      bool ok = true;
      double d;
      if (key == "tend") ok = to_double(val, &cfg->tEnd);
      else if (key == "nstepmax") ok = to_int(val, &cfg->nStepmax);
      else if (key == "noutput") ok = to_int(val, &cfg->nOutput);
      else if (key == "nx") ok = to_int(val, &cfg->p.nx);
      else if (key == "ny") ok = to_int(val, &cfg->p.ny);
      else if (key == "boundary_type_xmin") ok = to_int(val, &cfg->p.boundary_type_xmin);
      else if (key == "boundary_type_xmax") ok = to_int(val, &cfg->p.boundary_type_xmax);
      else if (key == "boundary_type_ymin") ok = to_int(val, &cfg->p.boundary_type_ymin);
      else if (key == "boundary_type_ymax") ok = to_int(val, &cfg->p.boundary_type_ymax);
      else if (key == "gamma0") ok = to_double(val, &cfg->p.gamma0);
      else if (key == "cfl") ok = to_double(val, &cfg->p.cfl);
      else if (key == "smallr") ok = to_double(val, &cfg->p.smallr);
      else if (key == "smallc") ok = to_double(val, &cfg->p.smallc);
      else if (key == "niter_riemann") ok = to_int(val, &cfg->p.niter_riemann);
      else if (key == "iorder") ok = to_int(val, &cfg->p.iorder);
      else if (key == "slope_type") {
        // integer in serial_ref, real in stdpar/cuf (m_HydroParameters.cuf:59)
        ok = to_int(val, &cfg->p.slope_type);
        if (!ok && to_double(val, &d) && d == (double)(int)d) { cfg->p.slope_type = (int)d; ok = true; }
      } else if (key == "implementationversion") ok = to_int(val, &cfg->p.implementation_version);
      else if (key == "precision") ok = to_int(val, &cfg->p.precision);
      else if (key == "riemann_solver") {
        std::string v = lower(unquote(val));
        if (v == "approx" || v == "0") cfg->p.riemann_solver = E2D_RIEMANN_APPROX;
        else if (v == "hllc" || v == "2") cfg->p.riemann_solver = E2D_RIEMANN_HLLC;
        else ok = false;
      }
      if (!ok) return "bad value '" + val + "' for " + key;
    }
  }
  if (cfg->p.implementation_version < 0 || cfg->p.implementation_version > 2)
    return "The implementation version parameter should 0, 1 or 2 !!! Check your namelist file, section OTHER";
  if (cfg->nOutput <= 0) return "nOutput must be positive";
  return std::string();
}
