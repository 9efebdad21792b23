// Autotune table: load, save, lookup (see Autotune in igr_engine.h).
#include <cstdio>
#include <fstream>
#include <sstream>

#include "igr_engine.h"

namespace igrgpu {

void Autotune::load() {
  if (path.empty()) return;
  std::ifstream in(path);
  if (!in) return;  // no cache yet
  std::string line;
  while (std::getline(in, line)) {
    if (line.empty() || line[0] == '#') continue;
    const size_t tab = line.find('\t');
    if (tab == std::string::npos) continue;
    try {
      table[line.substr(0, tab)] = std::stoi(line.substr(tab + 1));
    } catch (...) {
      // a malformed line is skipped; the entry is measured again
    }
  }
}

void Autotune::save() const {
  if (path.empty()) return;
  const std::string tmp = path + ".tmp";
  {
    std::ofstream out(tmp, std::ios::trunc);
    if (!out) throw Error(1, "cannot write autotune cache " + tmp);
    out << "# libigr_gb300 autotune cache: key<TAB>value\n";
    for (const auto& kv : table) out << kv.first << '\t' << kv.second << '\n';
    if (!out) throw Error(1, "cannot write autotune cache " + tmp);
  }
  if (std::rename(tmp.c_str(), path.c_str()) != 0) throw Error(1, "cannot replace autotune cache " + path);
}

bool Autotune::get(const std::string& key, int* v) const {
  const auto it = table.find(key);
  if (it == table.end()) return false;
  *v = it->second;
  return true;
}

void Autotune::put(const std::string& key, int v) {
  table[key] = v;
  try {
    save();
  } catch (const Error&) {
    // the cache file became unwritable after igr_set_autotune checked it:
    // keep the entry in memory and let the solve finish
  }
}

}  // namespace igrgpu
