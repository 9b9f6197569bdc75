// mm_options(): the reference's "key=value, key value" option grammar
// (src/sff/mm_options.l:18-97, mm_options() at mm_options.l:276).
//
// Items are separated by blanks, tabs, newlines or commas; a key is joined
// to its value by "=" (blanks allowed around it) or by blanks alone.  Every
// accepted item is echoed as "\tmm_options:  <item>" to nabout
// (mm_options.l:8) and settings are cumulative across calls.  An unknown key
// or a value outside the key's accepted set prints an error and exits, as
// the reference does (mm_options.l:99-111).  Keys beginning "sffg_" are this
// library's own and select device-side behaviour.
#include "sffg_internal.h"

#include <cctype>
#include <chrono>
#include <cstdlib>
#include <cstring>
#include <functional>

// The caller normally defines nabout (the reference requires it, e.g.
// test/tmd.c:18).  A weak definition lets processes that do not (Python via
// ctypes) load the library; the caller's strong definition takes precedence.
extern "C" {
__attribute__((weak)) FILE *nabout = nullptr;
}

namespace sffg {

Options &options() {
  static Options o;
  return o;
}

FILE *legacy_out() { return nabout ? nabout : stdout; }

Timers &timers() {
  static Timers t;
  return t;
}

double wall_seconds() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

namespace {

[[noreturn]] void option_error(const std::string &item) {
  std::fprintf(stderr, "Error: mm_option: unknown keyword or invalid value: %s\n", item.c_str());
  std::exit(1);
}

bool parse_double(const std::string &v, double &out) {
  char *end = nullptr;
  out = std::strtod(v.c_str(), &end);
  return end && *end == '\0' && end != v.c_str();
}

bool parse_int(const std::string &v, long long &out) {
  char *end = nullptr;
  out = std::strtoll(v.c_str(), &end, 10);
  return end && *end == '\0' && end != v.c_str();
}

struct Key {
  const char *name;
  std::function<bool(Options &, const std::string &)> set;
};

auto dbl(double Options::*m) {
  return [m](Options &o, const std::string &v) {
    double d;
    if (!parse_double(v, d)) return false;
    o.*m = d;
    return true;
  };
}

// Integer keys; lo/hi bound the values the reference's patterns accept.
auto integer(int Options::*m, long long lo, long long hi, bool zero_means_never = false) {
  return [=](Options &o, const std::string &v) {
    long long d;
    if (!parse_int(v, d) || d < lo || d > hi) return false;
    o.*m = static_cast<int>(d);
    if (zero_means_never && d == 0) o.*m = 9999999;
    return true;
  };
}

auto choice(int Options::*m, std::initializer_list<int> allowed) {
  std::vector<int> ok(allowed);
  return [=](Options &o, const std::string &v) {
    long long d;
    if (!parse_int(v, d)) return false;
    for (int a : ok)
      if (a == d) {
        o.*m = static_cast<int>(d);
        return true;
      }
    return false;
  };
}

const std::vector<Key> &keys() {
  static const std::vector<Key> k = {
      {"cut", dbl(&Options::cut)},
      {"cutnp", dbl(&Options::cutnp)},
      {"scnb", dbl(&Options::scnb)},
      {"scee", dbl(&Options::scee)},
      {"ntpr", integer(&Options::ntpr, 1, 1LL << 31, true)},
      {"hcp", choice(&Options::hcp, {0, 1, 2, 4})},
      {"hcp_h1", dbl(&Options::hcp_h1)},
      {"hcp_h2", dbl(&Options::hcp_h2)},
      {"hcp_h3", dbl(&Options::hcp_h3)},
      {"dhcp", dbl(&Options::dhcp)},
      {"nscm", integer(&Options::nscm, 0, 1LL << 31)},
      {"nsnb", integer(&Options::nsnb, 0, 1LL << 31)},
      {"nsnp", integer(&Options::nsnp, 0, 1LL << 31)},
      {"ntwx", integer(&Options::ntwx, 0, 1LL << 31)},
      {"nchk", integer(&Options::nchk, 0, 1LL << 31)},
      {"nchk2", integer(&Options::nchk2, 0, 1LL << 31)},
      {"dt", dbl(&Options::dt)},
      {"t", dbl(&Options::t)},
      {"tautp", dbl(&Options::tautp)},
      {"temp0", dbl(&Options::temp0)},
      {"tempi", dbl(&Options::tempi)},
      {"vlimit", dbl(&Options::vlimit)},
      {"gamma_ln", dbl(&Options::gamma_ln)},
      {"genmass", dbl(&Options::genmass)},
      {"wcons", dbl(&Options::wcons)},
      {"ntpr_md", integer(&Options::ntpr_md, 1, 1LL << 31, true)},
      {"zerov", integer(&Options::zerov, 0, 1LL << 31)},
      {"k4d", dbl(&Options::k4d)},
      {"ips", choice(&Options::ips, {0, 1, 2, 3})},
      {"gb", choice(&Options::gb, {0, 1, 2, 3, 5, 7, 8})},
      {"gb_debug", choice(&Options::gb_debug, {0, 1})},
      {"nr_debug", choice(&Options::nr_debug, {0, 1})},
      {"gb2_debug", choice(&Options::gb2_debug, {0, 1})},
      {"gbsa_debug", choice(&Options::gbsa_debug, {0, 1})},
      {"e_debug", choice(&Options::e_debug, {0, 1, 2, 3})},
      {"epsext", dbl(&Options::epsext)},
      {"kappa", dbl(&Options::kappa)},
      {"rgbmax", dbl(&Options::rgbmax)},
      {"surften", dbl(&Options::surften)},
      {"dradius", dbl(&Options::dradius)},
      {"deltar", dbl(&Options::deltar)},
      {"rwater", dbl(&Options::rwater)},
      {"alphanp", dbl(&Options::alphanp)},
      {"kappanp", dbl(&Options::kappanp)},
      {"min_volume", dbl(&Options::min_volume)},
      {"max_set_size", integer(&Options::max_set_size, 0, 1LL << 31)},
      {"MPI_min_tasks", integer(&Options::mpi_min_tasks, 0, 1LL << 31)},
      {"cull_np_lists", choice(&Options::cull_np_lists, {0, 1})},
      {"use_lower_tri", choice(&Options::use_lower_tri, {0, 1})},
      {"dynamic_loops", choice(&Options::dynamic_loops, {0, 1})},
      {"blocksize", integer(&Options::blocksize, 0, 1LL << 31)},
      {"gbsa", choice(&Options::gbsa, {0, 1})},
      {"dim", choice(&Options::dim, {3, 4})},
      {"dielc", dbl(&Options::dielc)},
      {"rattle", choice(&Options::irattle, {0, 1, 2})},
      {"diel",
       [](Options &o, const std::string &v) {
         static const std::pair<const char *, int> m[] = {
             {"Yammp", -5}, {"R94", -4}, {"RL94", -3}, {"RL", -2}, {"R", 0}, {"C", 1}};
         for (auto &e : m)
           if (v == e.first) {
             o.dield = e.second;
             return true;
           }
         return false;
       }},
      {"sffg_noise",
       [](Options &o, const std::string &v) {
         if (v == "reference") o.sffg_noise = 0;
         else if (v == "philox") o.sffg_noise = 1;
         else return false;
         return true;
       }},
      {"sffg_seed",
       [](Options &o, const std::string &v) {
         long long d;
         if (!parse_int(v, d)) return false;
         o.sffg_seed = static_cast<unsigned long long>(d);
         return true;
       }},
      {"sffg_graph", choice(&Options::sffg_graph, {0, 1})},
      {"sffg_tune", choice(&Options::sffg_tune, {0, 1})},
      {"sffg_lj_shared", choice(&Options::sffg_lj_shared, {0, 1})},
      {"sffg_serve_classes", choice(&Options::sffg_serve_classes, {0, 1})},
      {"sffg_verbose", choice(&Options::sffg_verbose, {0, 1})},
  };
  return k;
}

}  // namespace

// Parses opts into o; echoes each item when echo is set.  Returns 0, or -1
// with the offending item in *bad when fail_stop is false.
int parse_options(const char *opts, Options &o, bool echo, bool fail_stop, std::string *bad) {
  const char *p = opts ? opts : "";
  auto is_sep = [](char c) { return c == ' ' || c == ',' || c == '\t' || c == '\n'; };
  while (*p) {
    while (*p && is_sep(*p)) p++;
    if (!*p) break;
    const char *start = p;
    while (std::isalnum(static_cast<unsigned char>(*p)) || *p == '_') p++;
    std::string key(start, p);
    while (*p == ' ') p++;
    if (*p == '=') {
      p++;
      while (*p == ' ') p++;
    }
    const char *vs = p;
    while (*p && !is_sep(*p)) p++;
    std::string val(vs, p), item(start, p);
    bool ok = false;
    if (!key.empty() && !val.empty()) {
      for (const Key &k : keys())
        if (key == k.name) {
          ok = k.set(o, val);
          break;
        }
    }
    if (!ok) {
      if (fail_stop) option_error(item.empty() ? std::string(start) : item);
      if (bad) *bad = item.empty() ? std::string(start) : item;
      return -1;
    }
    if (echo) std::fprintf(legacy_out(), "\tmm_options:  %s\n", item.c_str());
  }
  return 0;
}

}  // namespace sffg

extern "C" void sffg_options_reset(void) { sffg::options() = sffg::Options(); }

extern "C" INT_T mm_options(STRING_T *opts) {
  sffg::parse_options(opts, sffg::options(), true, true, nullptr);
  return 0;
}
