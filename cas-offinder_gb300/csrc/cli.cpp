// cas-offinder: drop-in command line for the GB300 engine.
//
// Same argv and files as the reference (main.cpp:72-157):
//   cas-offinder [--summary file] {input_filename|-} {C|G|A}[device_id(s)] {output_filename|-}
// Line 1 of the input names a FASTA/2BIT file or a directory, which is walked
// in readdir order taking regular files and symlinks (main.cpp:133-147).  The
// output starts with the reference's two header lines (writeHeaders,
// cas-offinder.cpp:319-328), then the rows of each genome file.  All work runs
// on one CUDA device through libcasoff.so; the device letter is accepted for
// compatibility and the first listed id (default 0) is the CUDA ordinal.  An
// output file name ending in ".gz" gets the same text gzip-compressed
// (cof_gzip_*, blocks deflated on all host cores).
#include <dirent.h>
#include <sys/stat.h>
#include <sys/time.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <iterator>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/cof.h"

namespace {

void usage() {
  std::cout << "Cas-OFFinder 3.0.0 (GB300 engine)\n\n"
               "Usage: cas-offinder [options] {input_filename|-} {C|G|A}[device_id(s)] {output_filename|-}\n"
               "(all letters run on the CUDA device given by the first id, default 0)\n\n"
               "Options\n"
               "  --summary <file>\t\t\t Print summary table to the specified file.\n\n"
               "Example input file (DNA bulge 2, RNA bulge 1):\n"
               "/var/chromosomes/human_grch38\n"
               "NNNNNNNNNNNNNNNNNNNNNRG 2 1\n"
               "GGCCGACCTGTCGCTGACGCNNN 5\n"
               "CGCCAGCGTCAGCGACAGGTNNN 5\n"
               "ACGGCGCCAGCGTCAGCGACNNN 5\n"
               "GTCGCTGACGCTGGCGCCGTNNN 5\n";
}

// First device id of a "0,1" / "0:4[:step]" list (Cas_OFFinder::Cas_OFFinder,
// cas-offinder.cpp:131-156); 0 when none is given.
int first_device(const std::string& arg) {
  if (arg.empty()) return 0;
  std::string first = arg.substr(0, arg.find(','));
  first = first.substr(0, first.find(':'));
  return atoi(first.c_str());
}

bool write_all(FILE* f, const char* p, size_t n) { return fwrite(p, 1, n, f) == n; }

}  // namespace

int main(int argc, char** argv) {
  struct timeval t0, t1;
  gettimeofday(&t0, nullptr);
  std::vector<std::string> pos;
  std::string summary_path;
  for (int i = 1; i < argc; ++i) {
    std::string a = argv[i];
    if (a.size() > 2 && a[0] == '-' && a[1] == '-') {
      if (a.substr(2) == "summary" && i + 1 < argc) {
        summary_path = argv[++i];
      } else {
        usage();
        return 0;
      }
    } else {
      pos.push_back(a);
    }
  }
  if (pos.size() < 3) {
    usage();
    return 0;
  }
  const char letter = pos[1].empty() ? 0 : pos[1][0];
  if (letter != 'C' && letter != 'G' && letter != 'A') {
    std::cerr << "Unknown option: " << pos[1] << std::endl;
    return 1;
  }
  const int device = first_device(pos[1].substr(1));

  cof_handle* h = nullptr;
  if (cof_open(device, &h) != COF_OK) {
    std::cerr << "No CUDA device available: " << cof_open_error() << std::endl;
    return 1;
  }
  std::cerr << "Loading input file..." << std::endl;
  std::string input;
  if (pos[0] == "-") {
    input.assign(std::istreambuf_iterator<char>(std::cin), std::istreambuf_iterator<char>());
  } else {
    std::ifstream f(pos[0], std::ios::binary);
    if (!f.good()) {
      std::cerr << "Critical error! Cannot read input file." << std::endl;
      return 1;
    }
    input.assign(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
  }
  if (cof_read_input(h, input.data(), input.size()) != COF_OK) {
    std::cerr << "Critical error! " << cof_last_error(h) << std::endl;
    return 1;
  }
  if (!summary_path.empty()) cof_set_summary(h, 1);

  FILE* out = stdout;
  cof_gzip* gz = nullptr;
  const bool gzip = pos[2].size() > 3 && pos[2].compare(pos[2].size() - 3, 3, ".gz") == 0;
  if (gzip) {
    const cof_status st = cof_gzip_open(pos[2].c_str(), 1, 0, &gz);
    if (st != COF_OK) {
      std::cerr << (st == COF_ERR_UNSUPPORTED ? "No zlib for gzip output " : "Cannot open output file ") << pos[2]
                << std::endl;
      return 1;
    }
  } else if (pos[2] != "-") {
    out = fopen(pos[2].c_str(), "wb");
    if (!out) {
      std::cerr << "Cannot open output file " << pos[2] << std::endl;
      return 1;
    }
  }
  // Rows are written as they come off the GPU, chunk by chunk.
  cof_write_fn writer = gz ? cof_gzip_write_fn : [](void* ctx, const char* data, size_t n) -> int {
    return write_all((FILE*)ctx, data, n) ? 0 : 1;
  };
  void* wctx = gz ? (void*)gz : (void*)out;
  const char* header = cof_header_text();
  writer(wctx, header, strlen(header));
  if (!gz) fflush(out);

  int failed = 0;
  auto run_file = [&](const std::string& path) {
    std::cerr << "Reading " << path << "..." << std::endl;
    cof_status st = cof_genome_load_file(h, path.c_str());
    if (st == COF_ERR_NOT_GENOME) {
      std::cerr << "Skipping non-acceptable file " << path << "..." << std::endl;
      return;
    }
    if (st != COF_OK) {
      std::cerr << "Error loading " << path << ": " << cof_last_error(h) << std::endl;
      failed = 1;
      return;
    }
    if ((st = cof_search_stream(h, writer, wctx, nullptr)) != COF_OK) {
      if (st == COF_ERR_IO) std::cerr << "Write error on " << pos[2] << std::endl;
      else std::cerr << "Search failed on " << path << ": " << cof_last_error(h) << std::endl;
      failed = 1;
      return;
    }
    if (!gz) fflush(out);
    if (!summary_path.empty()) {
      std::cerr << "Writing summary file..." << std::endl;
      const char* text = nullptr;
      size_t tl = 0;
      cof_summary_text(h, &text, &tl);
      if (summary_path == "-") {
        write_all(stdout, text, tl);
        fflush(stdout);
      } else {
        FILE* sf = fopen(summary_path.c_str(), "wb");
        if (sf) {
          write_all(sf, text, tl);
          fclose(sf);
        }
      }
    }
  };

  const std::string target = cof_genome_path(h);
  if (DIR* dir = opendir(target.c_str())) {
    while (dirent* e = readdir(dir)) {
      if (e->d_type == DT_REG || e->d_type == DT_LNK) run_file(target + "/" + e->d_name);
      if (failed) break;
    }
    closedir(dir);
  } else {
    struct stat st;
    if (stat(target.c_str(), &st) != 0) {
      std::cerr << "An error has occured while opening directory: " << target << std::endl;
      return 1;
    }
    run_file(target);
  }
  if (gz) {
    if (cof_gzip_close(gz) != COF_OK) {
      std::cerr << "Write error on " << pos[2] << std::endl;
      failed = 1;
    }
  } else if (out != stdout) {
    fclose(out);
  }
  cof_close(h);
  gettimeofday(&t1, nullptr);
  std::cerr << (float)((t1.tv_sec - t0.tv_sec) + (t1.tv_usec - t0.tv_usec) / 1e6) << " seconds elapsed." << std::endl;
  return failed;
}
