// clpixel_main.cpp -- standalone driver, the counterpart of
// IndependentEntrypoint.cpp:137-199.
//
//   clpixel <folder with .dat files> [number of files=50] [--dump DIR]
//
// Reads the .dat files (IndependentEntrypoint.cpp:89-123 container) round
// robin, runs independent_execute (sort + search) and
// independent_post_execute.  The file list is sorted by name, where the
// reference takes readdir order (:163-176), so runs are reproducible.
// --dump writes one DIR/<i>.out per event in the reference's printTrack
// format (KernelInvoker.cpp:209-243,285-306), readable by the reference's
// tools/comparetracks.py.
#include <dirent.h>

#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <map>
#include <string>
#include <vector>

#include "../../include/GpuPixelSearchByTriplet.h"
#include "../../include/velo_search.h"

namespace {

bool read_dat(const std::string& path, std::vector<uint8_t>& out) {
  std::ifstream f(path, std::ios::binary);
  if (!f) return false;
  int32_t name_len = 0, size = 0;
  if (!f.read(reinterpret_cast<char*>(&name_len), 4) || name_len < 0) return false;
  f.seekg(name_len, std::ios::cur);
  if (!f.read(reinterpret_cast<char*>(&size), 4) || size < 0) return false;
  out.resize((size_t)size);
  return (bool)f.read(reinterpret_cast<char*>(out.data()), size);
}

int closest_module(int z, const std::map<int, int>& zmap) {   // KernelInvoker.cpp:314-335
  auto it = zmap.find(z);
  if (it != zmap.end()) return it->second;
  for (int err = 1; err < (1 << 20); ++err) {
    if ((it = zmap.find(z - err)) != zmap.end()) return it->second;
    if ((it = zmap.find(z + err)) != zmap.end()) return it->second;
  }
  return -1;
}

void dump_event(const std::string& path, const std::vector<uint8_t>& ev, const std::vector<uint8_t>& out) {
  int32_t S, H;
  std::memcpy(&S, ev.data(), 4);
  std::memcpy(&H, ev.data() + 4, 4);
  const int32_t* sz = reinterpret_cast<const int32_t*>(ev.data() + 8);
  const uint32_t* ids = reinterpret_cast<const uint32_t*>(ev.data() + 8 + 12 * S);
  const float* x = reinterpret_cast<const float*>(ids + H);
  const float* y = x + H;
  const float* z = y + H;
  std::map<int, int> zmap;
  for (int m = 0; m < S; ++m) zmap[sz[m]] = m;
  for (int h = 0; h < H; ++h) {
    const int zi = (int)z[h];
    if (!zmap.count(zi)) zmap[zi] = closest_module(zi, zmap);
  }
  std::ofstream os(path);
  const velo_track* t = reinterpret_cast<const velo_track*>(out.data());
  const size_t n = out.size() / sizeof(velo_track);
  for (size_t i = 0; i < n; ++i) {
    os << "Track #" << i << ", length " << (int)t[i].hitsNum << std::endl;
    for (uint32_t k = 0; k < t[i].hitsNum; ++k) {
      const uint32_t h = t[i].hits[k];
      os << " " << std::setw(8) << ids[h] << " (" << h << ")"
         << " module " << std::setw(2) << zmap.at((int)z[h]) << ", x " << std::setw(6) << x[h]
         << ", y " << std::setw(6) << y[h] << ", z " << std::setw(6) << z[h] << std::endl;
    }
    os << std::endl;
  }
}

}  // namespace

int main(int argc, char* argv[]) {
  std::string folder, dump_dir;
  size_t n_files = 50;   // IndependentEntrypoint.cpp:142
  int repeat = 1;        // > 1: run the batch again (steady state: context and buffers reused)
  std::vector<std::string> pos;
  for (int i = 1; i < argc; ++i) {
    if (std::strcmp(argv[i], "--dump") == 0 && i + 1 < argc) dump_dir = argv[++i];
    else if (std::strcmp(argv[i], "--repeat") == 0 && i + 1 < argc) repeat = std::max(1, std::atoi(argv[++i]));
    else pos.emplace_back(argv[i]);
  }
  if (pos.empty()) {
    std::cerr << "Usage: " << argv[0] << " <folder including .dat files> [number of files to process=50]"
              << " [--dump DIR] [--repeat K]" << std::endl;
    return -1;
  }
  folder = pos[0];
  if (pos.size() >= 2) n_files = (size_t)std::atoi(pos[1].c_str());
  std::cout << "Execution options:" << std::endl
            << " Executable: " << argv[0] << std::endl
            << " Folder name: " << folder << std::endl
            << " Number of files: " << n_files << std::endl << std::endl;
  std::vector<std::string> files;
  if (DIR* d = opendir(folder.c_str())) {
    while (dirent* ent = readdir(d)) {
      std::string f = ent->d_name;
      const size_t dot = f.find_last_of('.');
      if (dot != std::string::npos && f.substr(dot + 1) == "dat") files.push_back(f);
    }
    closedir(d);
  }
  if (files.empty()) {
    std::cerr << "Directory " << folder << " either could not be opened, or is empty" << std::endl;
    return -1;
  }
  std::sort(files.begin(), files.end());
  std::vector<std::vector<uint8_t>> input(n_files);
  for (size_t i = 0; i < n_files; ++i) {
    const std::string path = folder + "/" + files[i % files.size()];
    if (!read_dat(path, input[i])) {
      std::cerr << "Error: File " << path << " could not be read." << std::endl;
      return -1;
    }
  }
  std::cout << input.size() << " files read" << std::endl;
  std::vector<std::vector<uint8_t>> output;
  for (int r = 0; r < repeat; ++r) {
    output.clear();
    independent_execute(input, output);
  }
  if (!dump_dir.empty())
    for (size_t i = 0; i < output.size(); ++i)
      dump_event(dump_dir + "/" + std::to_string(i) + ".out", input[i], output[i]);
  independent_post_execute(output);
  return 0;
}
