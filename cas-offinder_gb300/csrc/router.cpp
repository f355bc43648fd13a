// Served mode over several resident genomes.
//
// The reference searches the genome that line 1 of each input file names: a
// file, or a directory whose files are read and searched one after another in
// readdir order, their rows written in that order (main.cpp:133-147).  A
// router keeps a set of such genomes resident on one device -- one handle and
// one server (server.cu) per genome file -- and sends each request to the
// servers of the genome its input file names, so requests for different
// genomes run side by side and a request's rows are those of the CLI on that
// input file: the rows of each file of the set, in the set's file order.
#include <dirent.h>
#include <limits.h>
#include <stdlib.h>
#include <sys/stat.h>

#include <algorithm>
#include <chrono>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/cof.h"
#include "cof_internal.h"

namespace {

struct Member {
  std::string path;
  cof_handle* h = nullptr;
  cof_server* s = nullptr;
};

// The resident files of one genome path (one file, or a directory's files).
struct GenomeSet {
  std::string key;
  std::vector<Member> files;
  uint64_t outstanding = 0;  // submitted, not yet released
  ~GenomeSet() {
    for (Member& m : files) {
      if (m.s) cof_server_stop(m.s);
      if (m.h) cof_close(m.h);
    }
  }
};

struct Ticket {
  GenomeSet* set = nullptr;
  std::vector<uint64_t> sub;  // one server ticket per file of the set
  double t_submit = 0;
  bool joined = false;
  std::string rows;  // concatenated rows when the set has more than one file
  const char* view = nullptr;
  size_t view_len = 0;
  double latency_ms = 0;
};

double now_ms() {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// The set key: the path with symbolic links and relative parts resolved when
// it exists, else as written.
std::string genome_key(const std::string& path) {
  char buf[PATH_MAX];
  if (realpath(path.c_str(), buf)) return std::string(buf);
  return path;
}

}  // namespace

struct cof_router {
  int device = 0;
  uint64_t max_active_variants = 0, hit_buffer_bytes = 0, segment_positions = 0;
  bool auto_load = false;
  std::mutex mu;       // sets, tickets, last_error
  std::mutex load_mu;  // one genome load at a time
  std::map<std::string, std::unique_ptr<GenomeSet>> sets;
  std::unordered_map<uint64_t, std::shared_ptr<Ticket>> tickets;
  uint64_t next_ticket = 1;
  std::string last_error;
};

namespace {

cof_status rfail(cof_router* r, cof_status st, const std::string& msg) {
  std::lock_guard<std::mutex> lock(r->mu);
  r->last_error = msg;
  return st;
}

// Opens a handle, loads one genome file and starts its server.
cof_status open_member(cof_router* r, const std::string& path, Member& m, std::string& err) {
  m.path = path;
  cof_status st = cof_open(r->device, &m.h);
  if (st != COF_OK) {
    err = "cannot open device " + std::to_string(r->device);
    return st;
  }
  if ((st = cof_genome_load_file(m.h, path.c_str())) != COF_OK) {
    err = cof_last_error(m.h);
    return st;
  }
  if ((st = cof_server_start(m.h, r->max_active_variants, r->hit_buffer_bytes, r->segment_positions, &m.s)) !=
      COF_OK) {
    err = cof_last_error(m.h);
    return st;
  }
  return COF_OK;
}

// Loads the genome path as the CLI reads it: every regular file (or link) of
// a directory in readdir order, files that are neither FASTA nor 2BIT
// skipped; else the one file.
cof_status load_set(cof_router* r, const std::string& path, std::unique_ptr<GenomeSet>& out, std::string& err) {
  auto set = std::make_unique<GenomeSet>();
  set->key = genome_key(path);
  std::vector<std::string> files;
  if (DIR* dir = opendir(path.c_str())) {
    while (dirent* e = readdir(dir))
      if (e->d_type == DT_REG || e->d_type == DT_LNK) files.push_back(path + "/" + e->d_name);
    closedir(dir);
  } else {
    struct stat st;
    if (stat(path.c_str(), &st) != 0) {
      err = "An error has occured while opening directory: " + path;
      return COF_ERR_IO;
    }
    files.push_back(path);
  }
  for (const std::string& f : files) {
    Member m;
    cof_status st = open_member(r, f, m, err);
    if (st == COF_ERR_NOT_GENOME) {
      if (m.h) cof_close(m.h);
      continue;
    }
    set->files.push_back(m);  // closed with the set on failure
    if (st != COF_OK) {
      err = "loading " + f + ": " + err;
      return st;
    }
  }
  out = std::move(set);
  return COF_OK;
}

}  // namespace

extern "C" {

cof_status cof_router_open(int device, uint64_t max_active_variants, uint64_t hit_buffer_bytes,
                           uint64_t segment_positions, int auto_load, cof_router** out) {
  if (!out) return COF_ERR_ARG;
  cof_router* r = new cof_router();
  r->device = device;
  r->max_active_variants = max_active_variants;
  r->hit_buffer_bytes = hit_buffer_bytes;
  r->segment_positions = segment_positions;
  r->auto_load = auto_load != 0;
  *out = r;
  return COF_OK;
}

cof_status cof_router_add_genome(cof_router* r, const char* path, uint32_t* n_files) {
  if (!r || !path) return COF_ERR_ARG;
  std::lock_guard<std::mutex> load(r->load_mu);
  const std::string key = genome_key(path);
  {
    std::lock_guard<std::mutex> lock(r->mu);
    auto it = r->sets.find(key);
    if (it != r->sets.end()) {
      if (n_files) *n_files = (uint32_t)it->second->files.size();
      return COF_OK;
    }
  }
  std::unique_ptr<GenomeSet> set;
  std::string err;
  cof_status st = load_set(r, path, set, err);
  if (st != COF_OK) return rfail(r, st, err);
  if (n_files) *n_files = (uint32_t)set->files.size();
  std::lock_guard<std::mutex> lock(r->mu);
  r->sets[key] = std::move(set);
  return COF_OK;
}

cof_status cof_router_drop_genome(cof_router* r, const char* path) {
  if (!r || !path) return COF_ERR_ARG;
  std::unique_ptr<GenomeSet> gone;
  {
    std::lock_guard<std::mutex> lock(r->mu);
    auto it = r->sets.find(genome_key(path));
    if (it == r->sets.end()) {
      r->last_error = std::string("genome not resident: ") + path;
      return COF_ERR_STATE;
    }
    if (it->second->outstanding) {
      r->last_error = std::string("genome has requests not released: ") + path;
      return COF_ERR_STATE;
    }
    gone = std::move(it->second);
    r->sets.erase(it);
  }
  return COF_OK;  // servers stopped and handles closed outside the lock
}

cof_status cof_router_genomes(cof_router* r, uint32_t* n_sets, uint32_t* n_files) {
  if (!r) return COF_ERR_ARG;
  std::lock_guard<std::mutex> lock(r->mu);
  uint32_t f = 0;
  for (auto& kv : r->sets) f += (uint32_t)kv.second->files.size();
  if (n_sets) *n_sets = (uint32_t)r->sets.size();
  if (n_files) *n_files = f;
  return COF_OK;
}

cof_status cof_router_submit(cof_router* r, const char* text, size_t len, uint64_t* ticket) {
  if (!r || (!text && len) || !ticket) return COF_ERR_ARG;
  cof::Job job;
  std::string err;
  if (!cof::parse_job(text ? text : "", len, job, err)) return rfail(r, COF_ERR_INPUT, err);
  const std::string key = genome_key(job.genome_path);
  GenomeSet* set = nullptr;
  {
    std::lock_guard<std::mutex> lock(r->mu);
    auto it = r->sets.find(key);
    if (it != r->sets.end()) set = it->second.get(), ++set->outstanding;
  }
  if (!set) {
    if (!r->auto_load) return rfail(r, COF_ERR_STATE, "genome not resident: " + job.genome_path);
    cof_status st = cof_router_add_genome(r, job.genome_path.c_str(), nullptr);
    if (st != COF_OK) return st;
    std::lock_guard<std::mutex> lock(r->mu);
    auto it = r->sets.find(key);
    if (it == r->sets.end()) {  // dropped again meanwhile
      r->last_error = "genome not resident: " + job.genome_path;
      return COF_ERR_STATE;
    }
    set = it->second.get();
    ++set->outstanding;
  }
  auto t = std::make_shared<Ticket>();
  t->set = set;
  t->t_submit = now_ms();
  for (Member& m : set->files) {
    uint64_t sub = 0;
    cof_status st = cof_server_submit(m.s, text, len, &sub);
    if (st != COF_OK) {
      const std::string msg = cof_server_last_error(m.s);
      // Every file parses the same text, so this is rare (a server stopping):
      // the files that took the request finish it before it is dropped.
      for (size_t i = 0; i < t->sub.size(); ++i) {
        const char* rows = nullptr;
        size_t n = 0;
        cof_server_wait(set->files[i].s, t->sub[i], -1, &rows, &n, nullptr);
        cof_server_release(set->files[i].s, t->sub[i]);
      }
      std::lock_guard<std::mutex> lock(r->mu);
      --set->outstanding;
      r->last_error = msg;
      return st;
    }
    t->sub.push_back(sub);
  }
  std::lock_guard<std::mutex> lock(r->mu);
  *ticket = r->next_ticket++;
  r->tickets[*ticket] = t;
  return COF_OK;
}

cof_status cof_router_wait(cof_router* r, uint64_t ticket, int timeout_ms, const char** rows, size_t* rows_len,
                           double* latency_ms) {
  if (!r || !rows || !rows_len) return COF_ERR_ARG;
  std::shared_ptr<Ticket> t;
  {
    std::lock_guard<std::mutex> lock(r->mu);
    auto it = r->tickets.find(ticket);
    if (it == r->tickets.end()) {
      r->last_error = "unknown ticket " + std::to_string(ticket);
      return COF_ERR_ARG;
    }
    t = it->second;
  }
  if (!t->joined) {
    const double deadline = timeout_ms < 0 ? 0 : now_ms() + timeout_ms;
    std::vector<const char*> parts(t->sub.size());
    std::vector<size_t> lens(t->sub.size());
    double lat = 0;
    for (size_t i = 0; i < t->sub.size(); ++i) {
      int left = -1;
      if (timeout_ms >= 0) left = (int)std::max(0.0, deadline - now_ms());
      double l = 0;
      cof_status st = cof_server_wait(t->set->files[i].s, t->sub[i], left, &parts[i], &lens[i], &l);
      if (st != COF_OK) {
        if (st != COF_ERR_TIMEOUT) return rfail(r, st, cof_server_last_error(t->set->files[i].s));
        return st;
      }
      lat = std::max(lat, l);
    }
    if (parts.size() == 1) {
      t->view = parts[0], t->view_len = lens[0];
    } else {
      size_t total = 0;
      for (size_t n : lens) total += n;
      t->rows.reserve(total);
      for (size_t i = 0; i < parts.size(); ++i) t->rows.append(parts[i], lens[i]);
      t->view = t->rows.data(), t->view_len = t->rows.size();
    }
    t->latency_ms = parts.empty() ? now_ms() - t->t_submit : lat;
    t->joined = true;
  }
  *rows = t->view ? t->view : "";
  *rows_len = t->view_len;
  if (latency_ms) *latency_ms = t->latency_ms;
  return COF_OK;
}

cof_status cof_router_release(cof_router* r, uint64_t ticket) {
  if (!r) return COF_ERR_ARG;
  std::shared_ptr<Ticket> t;
  {
    std::lock_guard<std::mutex> lock(r->mu);
    auto it = r->tickets.find(ticket);
    if (it == r->tickets.end()) {
      r->last_error = "unknown ticket " + std::to_string(ticket);
      return COF_ERR_ARG;
    }
    t = it->second;
    if (!t->joined) {  // as cof_server_release: only a finished request
      r->last_error = "ticket " + std::to_string(ticket) + " has not been waited for";
      return COF_ERR_ARG;
    }
    r->tickets.erase(it);
  }
  for (size_t i = 0; i < t->sub.size(); ++i) cof_server_release(t->set->files[i].s, t->sub[i]);
  std::lock_guard<std::mutex> lock(r->mu);
  --t->set->outstanding;
  return COF_OK;
}

const char* cof_router_last_error(cof_router* r) {
  if (!r) return "";
  std::lock_guard<std::mutex> lock(r->mu);
  return r->last_error.c_str();
}

void cof_router_close(cof_router* r) {
  if (!r) return;
  {
    std::lock_guard<std::mutex> lock(r->mu);
    r->tickets.clear();
  }
  r->sets.clear();  // stops every server, closes every handle
  delete r;
}

}  // extern "C"
