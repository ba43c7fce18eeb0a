// Command-line plumbing shared by gmm_adapt and gmm_loglike: the option syntax of the reference's
// tools (boost::program_options: "--name value", "--name=value", "-x value", implicit booleans,
// repeatable options, an INI file given by -c whose values the command line overrides), their
// file-list rules and their output-file naming. Header-only; host code, no device work.
#pragma once

#include <dirent.h>
#include <sys/stat.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <fstream>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace gmmgb {
namespace cli {

// One option: long name, optional one-letter alias, kind and help line.
enum Kind { STR, MULTI, FLAG };  // FLAG = boolean with implicit value true
struct Opt {
  std::string name;
  char alias;
  Kind kind;
  std::string def;  // default value as text ("" = none)
  std::string help;
};

class Parser {
 public:
  explicit Parser(std::vector<Opt> opts) : opts_(std::move(opts)) {}

  // Parses argv, then the configuration file named by "config" (if that option exists and was
  // given). Unknown options throw std::runtime_error.
  void parse(int argc, char** argv) {
    for (int a = 1; a < argc; ++a) {
      std::string k = argv[a], v;
      bool has_v = false;
      const Opt* o = nullptr;
      if (k.rfind("--", 0) == 0) {
        const size_t eq = k.find('=');
        if (eq != std::string::npos) {
          v = k.substr(eq + 1);
          has_v = true;
          k = k.substr(0, eq);
        }
        o = find(k.substr(2));
      } else if (k.size() >= 2 && k[0] == '-') {
        o = find_alias(k[1]);
        if (o && k.size() > 2) {
          v = k.substr(2);
          has_v = true;
        }
      }
      if (!o) throw std::runtime_error("unrecognised option '" + std::string(argv[a]) + "' (see -h)");
      if (o->kind == FLAG) {
        set(*o, has_v ? v : "1", cmd_);
        continue;
      }
      if (!has_v) {
        if (a + 1 >= argc) throw std::runtime_error("option '--" + o->name + "' requires a value");
        v = argv[++a];
      }
      set(*o, v, cmd_);
    }
    values_ = cmd_;
    if (find("config") && count("config")) read_config(get("config"));
  }

  bool count(const std::string& n) const { return values_.count(n) && !values_.at(n).empty(); }
  std::string get(const std::string& n) const {
    if (count(n)) return values_.at(n).back();
    const Opt* o = find(n);
    return o ? o->def : std::string();
  }
  std::vector<std::string> all(const std::string& n) const { return count(n) ? values_.at(n) : std::vector<std::string>(); }
  int get_int(const std::string& n) const { return std::stoi(get(n)); }
  unsigned get_uint(const std::string& n) const { return (unsigned)std::stoul(get(n)); }
  float get_float(const std::string& n) const { return std::stof(get(n)); }
  bool get_bool(const std::string& n) const {
    const std::string v = get(n);
    if (v == "1" || v == "true" || v == "yes" || v == "on") return true;
    if (v.empty() || v == "0" || v == "false" || v == "no" || v == "off") return false;
    throw std::runtime_error("option '--" + n + "': '" + v + "' is not a boolean");
  }

  void help(const char* title) const {
    std::printf("%s\n", title);
    for (const auto& o : opts_) {
      std::string lhs = "  --" + o.name + (o.alias ? std::string(" [ -") + o.alias + " ]" : std::string());
      if (o.kind != FLAG) lhs += " arg";
      if (!o.def.empty()) lhs += " (=" + o.def + ")";
      std::printf("%-40s %s\n", lhs.c_str(), o.help.c_str());
    }
  }

 private:
  using Values = std::map<std::string, std::vector<std::string>>;
  const Opt* find(const std::string& n) const {
    for (const auto& o : opts_)
      if (o.name == n) return &o;
    return nullptr;
  }
  const Opt* find_alias(char c) const {
    for (const auto& o : opts_)
      if (o.alias == c) return &o;
    return nullptr;
  }
  static void set(const Opt& o, const std::string& v, Values& into) {
    if (o.kind == MULTI) into[o.name].push_back(v);
    else into[o.name] = {v};
  }
  // "name = value  # comment" lines; values of options the command line set are ignored.
  void read_config(const std::string& path) {
    std::ifstream f(path);
    if (!f) throw std::runtime_error("configuration file " + path + " could not be opened");
    Values cfg;
    std::string ln;
    while (std::getline(f, ln)) {
      const size_t hash = ln.find('#');
      if (hash != std::string::npos) ln.erase(hash);
      const size_t eq = ln.find('=');
      if (eq == std::string::npos) continue;
      const std::string k = trim(ln.substr(0, eq)), v = trim(ln.substr(eq + 1));
      if (k.empty()) continue;
      const Opt* o = find(k);
      if (!o) throw std::runtime_error("unrecognised option '" + k + "' in " + path);
      set(*o, v, cfg);
    }
    for (auto& kv : cfg)
      if (!cmd_.count(kv.first)) values_[kv.first] = kv.second;
  }
  static std::string trim(const std::string& s) {
    const size_t a = s.find_first_not_of(" \t\r"), b = s.find_last_not_of(" \t\r");
    return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
  }
  std::vector<Opt> opts_;
  Values cmd_, values_;
};

inline bool is_file(const std::string& p) {
  struct stat st;
  return ::stat(p.c_str(), &st) == 0 && S_ISREG(st.st_mode);
}
inline bool is_dir(const std::string& p) {
  struct stat st;
  return ::stat(p.c_str(), &st) == 0 && S_ISDIR(st.st_mode);
}

// The file name without directory and extension (boost::filesystem::basename).
inline std::string basename_noext(const std::string& p) {
  const size_t s = p.find_last_of('/');
  std::string f = s == std::string::npos ? p : p.substr(s + 1);
  const size_t d = f.rfind('.');
  return d == std::string::npos || d == 0 ? f : f.substr(0, d);
}

// Output path of an input file (GetNewPathC, tools/usefull_funcs.h:205-227): the file name moved
// into `dir` (when given) with its extension replaced by `ext` (unless ext is ".*").
inline std::string new_path(const std::string& file, const std::string& dir, const std::string& ext) {
  const size_t s = file.rfind('/');
  std::string out = (dir.empty() ? std::string() : dir + "/") + (s == std::string::npos ? file : file.substr(s + 1));
  if (ext != ".*") {
    const size_t sl = out.rfind('/'), dot = out.rfind('.');
    if (dot == std::string::npos || (sl != std::string::npos && dot < sl)) out += ext;
    else out.replace(dot, out.size() - dot, ext);
  }
  return out;
}

// A list argument (ReadTestList, tools/usefull_funcs.h:229-271): a directory contributes its
// regular files whose names end with `ext` (every file for ".*" or ""), sorted by name; a file
// contributes one path per non-empty line.
inline void read_list(const std::string& p, const std::string& ext, std::vector<std::string>* out) {
  if (is_dir(p)) {
    std::vector<std::string> names;
    if (DIR* d = ::opendir(p.c_str())) {
      while (dirent* e = ::readdir(d)) {
        const std::string n = e->d_name;
        if (n == "." || n == ".." || !is_file(p + "/" + n)) continue;
        if (ext.empty() || ext == ".*" || (n.size() >= ext.size() && n.compare(n.size() - ext.size(), ext.size(), ext) == 0))
          names.push_back(p + "/" + n);
      }
      ::closedir(d);
    } else {
      throw std::runtime_error("ReadTestList(): Reading of directory \"" + p + "\" content failed!");
    }
    std::sort(names.begin(), names.end());
    out->insert(out->end(), names.begin(), names.end());
    return;
  }
  std::ifstream f(p);
  std::string ln;
  while (std::getline(f, ln)) {
    if (!ln.empty() && ln.back() == '\r') ln.pop_back();
    if (!ln.empty()) out->push_back(ln);
  }
}

// saveMat (matrices/IOMats.h:169-227): text "x y\n", each value followed by a space, a newline per
// row and a final newline; binary int32 x, int32 y, then the floats.
inline void save_mat(const std::string& path, bool txt, const float* v, unsigned x, unsigned y) {
  FILE* f = std::fopen(path.c_str(), txt ? "w" : "wb");
  if (!f) throw std::runtime_error("saveMat(): file " + path + " could not be opened for writing");
  bool ok = true;
  if (txt) {
    ok = std::fprintf(f, "%u %u\n", x, y) > 0;
    for (unsigned i = 0; ok && i < x; ++i) {
      for (unsigned j = 0; ok && j < y; ++j) ok = std::fprintf(f, "%g ", v[(size_t)i * y + j]) > 0;
      ok = ok && std::fputc('\n', f) != EOF;
    }
    ok = ok && std::fputc('\n', f) != EOF;
  } else {
    const int32_t hx = (int32_t)x, hy = (int32_t)y;
    ok = std::fwrite(&hx, 4, 1, f) == 1 && std::fwrite(&hy, 4, 1, f) == 1 &&
         std::fwrite(v, sizeof(float), (size_t)x * y, f) == (size_t)x * y;
  }
  if (std::fclose(f) != 0 || !ok) throw std::runtime_error("saveMat(): Exception writing file " + path);
}

}  // namespace cli
}  // namespace gmmgb
