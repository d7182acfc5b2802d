// crg_tune.cu -- the autotuner's choices: an in-memory table, persisted to a
// small text file so that a later process starts with them.
//
// A choice is the index of the fastest candidate of one kernel family for one
// key (the device, the matrix copy's rows, columns and nonzeros, the field
// type and the field count; see crg_apply.cu for the families and their
// candidates).  Every candidate of a family computes the same bits, so a
// choice never changes a result.
//
// File: CRG_AUTOTUNE_CACHE if set ("" or "off": memory only), else
// $XDG_CACHE_HOME/crg_gb300/autotune.tsv, else $HOME/.cache/crg_gb300/autotune.tsv.
// One line per key: "<key>\t<choice>\t<milliseconds of each candidate>".
// Lines are appended (the last line of a key wins); a file that cannot be
// read or written leaves the table in memory.  CRG_AUTOTUNE=0 turns the tuner
// off (every family runs its first candidate, the defaults); CRG_AUTOTUNE_LOG=1
// prints each choice to stderr, marked "measured" or "cached".
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>

#include <map>
#include <mutex>
#include <string>

#include "crg_internal.cuh"

namespace crg {

namespace {

std::mutex g_tune_mu;
std::map<std::string, int>* g_tune = nullptr;  // key -> choice
bool g_tune_loaded = false;

std::string cache_path() {
  const char* e = getenv("CRG_AUTOTUNE_CACHE");
  if (e) return (strcmp(e, "off") == 0) ? std::string() : std::string(e);
  std::string base;
  if (const char* x = getenv("XDG_CACHE_HOME")) base = x;
  else if (const char* h = getenv("HOME")) base = std::string(h) + "/.cache";
  else return std::string();
  return base + "/crg_gb300/autotune.tsv";
}

void make_parent_dirs(const std::string& path) {
  for (size_t i = 1; i < path.size(); ++i)
    if (path[i] == '/') mkdir(path.substr(0, i).c_str(), 0755);  // existing directories: EEXIST, ignored
}

void load_locked() {
  if (g_tune_loaded) return;
  g_tune_loaded = true;
  if (!g_tune) g_tune = new std::map<std::string, int>();
  const std::string p = cache_path();
  if (p.empty()) return;
  FILE* f = fopen(p.c_str(), "r");
  if (!f) return;
  char line[1024];
  while (fgets(line, sizeof line, f)) {
    char* tab = strchr(line, '\t');
    if (!tab) continue;
    *tab = '\0';
    char* end = nullptr;
    const long c = strtol(tab + 1, &end, 10);
    if (end == tab + 1 || c < 0 || c > 64) continue;
    (*g_tune)[std::string(line)] = (int)c;
  }
  fclose(f);
}

bool log_on() {
  const char* e = getenv("CRG_AUTOTUNE_LOG");
  return e && strcmp(e, "0") != 0;
}

}  // namespace

bool tune_enabled() {
  const char* e = getenv("CRG_AUTOTUNE");
  return !(e && strcmp(e, "0") == 0);
}

bool tune_lookup(const std::string& key, int& choice) {
  std::lock_guard<std::mutex> lock(g_tune_mu);
  load_locked();
  auto it = g_tune->find(key);
  if (it == g_tune->end()) return false;
  choice = it->second;
  static std::map<std::string, bool>* logged = new std::map<std::string, bool>();
  if (log_on() && !(*logged)[key]) {
    (*logged)[key] = true;
    fprintf(stderr, "crg autotune: %s -> %d (cached)\n", key.c_str(), choice);
  }
  return true;
}

void tune_store(const std::string& key, int choice, const float* ms, int n) {
  std::lock_guard<std::mutex> lock(g_tune_mu);
  load_locked();
  (*g_tune)[key] = choice;
  std::string times;
  for (int i = 0; i < n; ++i) {
    char b[32];
    snprintf(b, sizeof b, "%s%.4f", i ? "," : "", ms[i]);
    times += b;
  }
  if (log_on()) fprintf(stderr, "crg autotune: %s -> %d (measured: %s ms)\n", key.c_str(), choice, times.c_str());
  const std::string p = cache_path();
  if (p.empty()) return;
  make_parent_dirs(p);
  FILE* f = fopen(p.c_str(), "a");
  if (!f) return;
  fprintf(f, "%s\t%d\t%s\n", key.c_str(), choice, times.c_str());
  fclose(f);
}

}  // namespace crg
