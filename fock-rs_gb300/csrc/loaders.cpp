// Host-side readers of the formats on either side of the path: xyz molecule
// files (chemfiles/src/xyz.rs:13-32) and MolSSI BSE JSON basis sets
// (basis_set/src/lib.rs:15-118), producing the fock_atom / fock_shell input
// of fock_ctx_create.  Plain C++ (no device code), so they also run on hosts
// without a GPU.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <regex>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/fock_gb300.h"

namespace {

// Element symbols H..Kr (Z = index + 1).
const char* const kSymbols[] = {"H",  "He", "Li", "Be", "B",  "C",  "N",  "O",  "F",  "Ne", "Na", "Mg",
                                "Al", "Si", "P",  "S",  "Cl", "Ar", "K",  "Ca", "Sc", "Ti", "V",  "Cr",
                                "Mn", "Fe", "Co", "Ni", "Cu", "Zn", "Ga", "Ge", "As", "Se", "Br", "Kr"};

int symbol_to_z(const std::string& s) {
  for (int z = 0; z < (int)(sizeof(kSymbols) / sizeof(kSymbols[0])); ++z)
    if (s == kSymbols[z]) return z + 1;
  return 0;
}

bool read_file(const char* path, std::string& out) {
  std::ifstream f(path, std::ios::binary);
  if (!f) return false;
  std::ostringstream ss;
  ss << f.rdbuf();
  out = ss.str();
  return true;
}

// ---------------------------------------------------------------------------
// A small JSON reader: objects, arrays, strings (with the common escapes),
// numbers, true/false/null.  Enough for BSE basis-set files.
// ---------------------------------------------------------------------------
struct JVal {
  enum Kind { NUL, BOOL, NUM, STR, ARR, OBJ } kind = NUL;
  double num = 0.0;
  bool b = false;
  std::string str;
  std::vector<JVal> arr;
  std::vector<std::pair<std::string, JVal>> obj;
  const JVal* get(const std::string& key) const {
    if (kind != OBJ) return nullptr;
    for (const auto& kv : obj)
      if (kv.first == key) return &kv.second;
    return nullptr;
  }
};

struct JParser {
  const std::string& s;
  size_t i = 0;
  explicit JParser(const std::string& text) : s(text) {}
  void ws() {
    while (i < s.size() && (s[i] == ' ' || s[i] == '\n' || s[i] == '\r' || s[i] == '\t')) ++i;
  }
  bool lit(const char* w) {
    const size_t n = std::strlen(w);
    if (s.compare(i, n, w) != 0) return false;
    i += n;
    return true;
  }
  bool string(std::string& out) {
    if (i >= s.size() || s[i] != '"') return false;
    ++i;
    out.clear();
    while (i < s.size() && s[i] != '"') {
      char ch = s[i++];
      if (ch == '\\') {
        if (i >= s.size()) return false;
        const char e = s[i++];
        switch (e) {
          case 'n': out += '\n'; break;
          case 't': out += '\t'; break;
          case 'r': out += '\r'; break;
          case 'b': out += '\b'; break;
          case 'f': out += '\f'; break;
          case 'u':  // keep the escape as text: basis files use it only in descriptions
            out += "\\u";
            break;
          default: out += e;
        }
      } else {
        out += ch;
      }
    }
    if (i >= s.size()) return false;
    ++i;
    return true;
  }
  bool value(JVal& v, int depth = 0) {
    if (depth > 64) return false;
    ws();
    if (i >= s.size()) return false;
    const char c = s[i];
    if (c == '{') {
      v.kind = JVal::OBJ;
      ++i;
      ws();
      if (i < s.size() && s[i] == '}') { ++i; return true; }
      for (;;) {
        ws();
        std::string key;
        if (!string(key)) return false;
        ws();
        if (i >= s.size() || s[i] != ':') return false;
        ++i;
        v.obj.emplace_back(key, JVal());
        if (!value(v.obj.back().second, depth + 1)) return false;
        ws();
        if (i < s.size() && s[i] == ',') { ++i; continue; }
        if (i < s.size() && s[i] == '}') { ++i; return true; }
        return false;
      }
    }
    if (c == '[') {
      v.kind = JVal::ARR;
      ++i;
      ws();
      if (i < s.size() && s[i] == ']') { ++i; return true; }
      for (;;) {
        v.arr.emplace_back();
        if (!value(v.arr.back(), depth + 1)) return false;
        ws();
        if (i < s.size() && s[i] == ',') { ++i; continue; }
        if (i < s.size() && s[i] == ']') { ++i; return true; }
        return false;
      }
    }
    if (c == '"') { v.kind = JVal::STR; return string(v.str); }
    if (lit("true")) { v.kind = JVal::BOOL; v.b = true; return true; }
    if (lit("false")) { v.kind = JVal::BOOL; v.b = false; return true; }
    if (lit("null")) { v.kind = JVal::NUL; return true; }
    char* end = nullptr;
    v.num = std::strtod(s.c_str() + i, &end);
    if (end == s.c_str() + i) return false;
    v.kind = JVal::NUM;
    i = (size_t)(end - s.c_str());
    return true;
  }
};

// A number given as a JSON string ("0.3425250914E+01", as BSE stores them) or number.
bool jnum(const JVal& v, double& out) {
  if (v.kind == JVal::NUM) { out = v.num; return true; }
  if (v.kind != JVal::STR) return false;
  char* end = nullptr;
  out = std::strtod(v.str.c_str(), &end);
  return end != v.str.c_str() && std::isfinite(out);
}

}  // namespace

extern "C" {

int fock_read_xyz(const char* path, fock_atom* atoms, int capacity, int* natom) {
  if (!path || !natom || capacity < 0 || (capacity > 0 && !atoms)) return FOCK_ERR_INVALID_ARG;
  std::string text;
  if (!read_file(path, text)) return FOCK_ERR_INVALID_ARG;
  // the reference's pattern, matched over the whole file (chemfiles/src/xyz.rs:14)
  static const std::regex pat(R"(\s*(\w+)\s+([+\-0-9.]+)\s+([+\-0-9.]+)\s+([0-9.+\-]+).*\b)");
  int n = 0;
  for (auto it = std::sregex_iterator(text.begin(), text.end(), pat); it != std::sregex_iterator(); ++it) {
    const std::smatch& m = *it;
    const int z = symbol_to_z(m[1].str());
    if (z == 0) return FOCK_ERR_INVALID_ARG;  // AtomType::from_symbol has no such element
    double x[3];
    for (int k = 0; k < 3; ++k) {
      char* end = nullptr;
      const std::string t = m[2 + k].str();
      x[k] = std::strtod(t.c_str(), &end);
      if (end == t.c_str()) return FOCK_ERR_INVALID_ARG;
    }
    if (n < capacity) atoms[n] = fock_atom{x[0] * 1.89, x[1] * 1.89, x[2] * 1.89, z};  // xyz.rs:24-26
    ++n;
  }
  *natom = n;
  return n > capacity ? FOCK_ERR_TOO_LARGE : FOCK_OK;
}

int fock_basis_shells(const char* json_path, const char* name, const fock_atom* atoms, int natom, fock_shell* shells,
                      int shell_capacity, double* exps, double* coefs, int prim_capacity, int* nshell, int* nprim) {
  if (!json_path || !atoms || natom <= 0 || !nshell || !nprim || shell_capacity < 0 || prim_capacity < 0 ||
      (shell_capacity > 0 && !shells) || (prim_capacity > 0 && (!exps || !coefs)))
    return FOCK_ERR_INVALID_ARG;
  std::string text;
  if (!read_file(json_path, text)) return FOCK_ERR_INVALID_ARG;
  JVal root;
  JParser parser(text);
  if (!parser.value(root) || root.kind != JVal::OBJ) return FOCK_ERR_INVALID_ARG;
  // a BSE file ({"elements": {...}, ...}), or a collection {name: BSE file or {Z: shells}}
  const JVal* set = &root;
  if (name && *name) {
    set = root.get(name);
    if (!set) return FOCK_ERR_INVALID_ARG;
  }
  const JVal* elements = set->get("elements");
  if (!elements) elements = set;
  if (elements->kind != JVal::OBJ) return FOCK_ERR_INVALID_ARG;
  int ns = 0, np = 0;
  for (int a = 0; a < natom; ++a) {
    const JVal* el = elements->get(std::to_string(atoms[a].Z));
    if (!el) return FOCK_ERR_INVALID_ARG;  // "Failed to get atom from basis set"
    const JVal* list = el->kind == JVal::OBJ ? el->get("electron_shells") : el;
    if (!list || list->kind != JVal::ARR) return FOCK_ERR_INVALID_ARG;
    for (const JVal& sh : list->arr) {
      const JVal* am = sh.get("angular_momentum");
      const JVal* ex = sh.get("exponents");
      const JVal* co = sh.get("coefficients");
      if (!am || !ex || !co || am->kind != JVal::ARR || ex->kind != JVal::ARR || co->kind != JVal::ARR)
        return FOCK_ERR_INVALID_ARG;
      const int k = (int)ex->arr.size();
      // one shell per angular momentum of the entry (SP entries give an s and a p
      // shell), coefficients row idx for angular momentum idx (basis_set/src/lib.rs:85-115)
      for (size_t idx = 0; idx < am->arr.size(); ++idx) {
        double lval = 0.0;
        if (!jnum(am->arr[idx], lval) || lval < 0 || idx >= co->arr.size()) return FOCK_ERR_INVALID_ARG;
        const JVal& crow = co->arr[idx];
        if (crow.kind != JVal::ARR || (int)crow.arr.size() != k || k == 0) return FOCK_ERR_INVALID_ARG;
        if (ns < shell_capacity && np + k <= prim_capacity) {
          for (int p = 0; p < k; ++p)
            if (!jnum(ex->arr[p], exps[np + p]) || !jnum(crow.arr[p], coefs[np + p])) return FOCK_ERR_INVALID_ARG;
          shells[ns] = fock_shell{(int)lval, k, a, exps + np, coefs + np};
        }
        ++ns;
        np += k;
      }
    }
  }
  *nshell = ns;
  *nprim = np;
  return (ns > shell_capacity || np > prim_capacity) ? FOCK_ERR_TOO_LARGE : FOCK_OK;
}

}  // extern "C"
