// Command-line front-end of the GB300 render path, a drop-in for the
// reference's `birp` program (src/main.cpp:24-317): the same flags, defaults,
// messages and output file names, rendering through the GPU classes.
//
//   -i file.dat | -i dir/   one cube, or every file of a directory (batch)
//   -c                      CMEM instead of a cube
//   -o prefix               output path prefix (FITS files <prefix><name>.fits)
//   -x -y -z  -a            spacecraft position and aim (x of the aim point)
//   -t                      trilinear interpolation (default nearest)
//   -s -h -w                pixel size and fields of view (degrees)
//   -v -b -d -p -q -r -f -e -g -u -j -k -l   CMEM parameters as the reference
//
// Extensions (no reference counterpart):
//   -m records|pairs|compact device layout of the cubes (default records)
//   -M n                    cubes rendered per GPU launch in batch mode (32)
//
// Batch mode differs from the reference in how it runs, not in what it
// writes: the directory's files are parsed on several host threads and each
// group of up to -M cubes is rendered in one batched launch (RenderBatch)
// instead of one render per cube; files are taken in name order (the
// reference's directory order is unspecified).
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdio>
#include <filesystem>
#include <iostream>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "birp/Camera.h"
#include "birp/Cmem.h"
#include "birp/DataCube.h"

namespace {

template <class T>
std::vector<T> explode(const std::string& s, char delim) {  // as Helper::explode_int / explode_float
  std::vector<T> out;
  std::stringstream ss(s);
  std::string item;
  while (std::getline(ss, item, delim)) {
    if (item.empty()) continue;
    if constexpr (std::is_same_v<T, int>) out.push_back(std::stoi(item));
    else out.push_back(std::stof(item));
  }
  return out;
}

bool ends_with(const std::string& s, const std::string& suffix) {
  return s.size() >= suffix.size() && s.compare(s.size() - suffix.size(), suffix.size(), suffix) == 0;
}

std::string base_name(const std::string& path) { return path.substr(path.find_last_of("/\\") + 1); }

}  // namespace

int main(int argc, char** argv) try {
  using namespace std::chrono;
  const auto start = high_resolution_clock::now();

  std::string input, output;
  bool have_mode = false, batch = false, use_cmem = false;
  // the reference's defaults (src/main.cpp:36-83)
  float pos_x = 5.91813f, pos_y = 6.74116f, pos_z = 17.7067f, aim = 7.81768f;
  bool interpolate = false;
  float pixel_size_deg = .25f, plot_fov_h = 36.f, plot_fov_w = 36.f;
  std::vector<int> v, b;
  std::vector<float> p = {1.f, 1.f, 3.f, 4.f};
  float dipole = 0, B = 0, alpha = 0, beta = 0, bs = 0, A1 = 0, A2 = 0, ay_bs = 0, az_bs = 0, density = 0;
  int layout = BIRP_CUBE_RECORDS;
  int per_launch = 32;

  int c;
  while ((c = getopt(argc, argv, "i:o:x:y:z:a:tcs:h:w:v:b:d:p:q:r:f:e:g:u:j:k:l:m:M:")) != -1) {
    switch (c) {
      case 'i':
        input = optarg;
        if (input.find(".dat") != std::string::npos) {
          batch = false;
          std::cout << "Using non-batch mode\n";
        } else if (ends_with(input, "/")) {
          batch = true;
          std::cout << "Using batch mode\n";
        } else {
          std::cout << "Please provide valid .dat datacube or use -c to use CMEM." << std::endl;
          return 3;
        }
        have_mode = true;
        break;
      case 'c': batch = false; use_cmem = true; have_mode = true; break;
      case 'o': output = optarg; break;
      case 'x': pos_x = std::stof(optarg); break;
      case 'y': pos_y = std::stof(optarg); break;
      case 'z': pos_z = std::stof(optarg); break;
      case 'a': aim = std::stof(optarg); break;
      case 't': interpolate = true; break;
      case 's': pixel_size_deg = std::stof(optarg); break;
      case 'h': plot_fov_h = std::stof(optarg); break;
      case 'w': plot_fov_w = std::stof(optarg); break;
      case 'v': v = explode<int>(optarg, ','); break;
      case 'b': b = explode<int>(optarg, ','); break;
      case 'd': dipole = std::stof(optarg); break;
      case 'p': p = explode<float>(optarg, ','); break;
      case 'q': B = std::stof(optarg); break;
      case 'r': alpha = std::stof(optarg); break;
      case 'f': beta = std::stof(optarg); break;
      case 'e': bs = std::stof(optarg); break;
      case 'g': A1 = std::stof(optarg); break;
      case 'u': A2 = std::stof(optarg); break;
      case 'j': ay_bs = std::stof(optarg); break;
      case 'k': az_bs = std::stof(optarg); break;
      case 'l': density = std::stof(optarg); break;
      case 'm':
        if (std::string(optarg) == "compact") layout = BIRP_CUBE_COMPACT;
        else if (std::string(optarg) == "pairs") layout = BIRP_CUBE_PAIRS;
        else if (std::string(optarg) == "records") layout = BIRP_CUBE_RECORDS;
        else throw std::invalid_argument("-m takes records, pairs or compact");
        break;
      case 'M': per_launch = std::max(1, std::stoi(optarg)); break;
      default: return 1;
    }
  }
  if (!have_mode) {
    std::cout << "Please provide valid .dat datacube or use -c to use CMEM." << std::endl;
    return 3;
  }

  if (batch) {
    std::vector<std::string> files;
    for (const auto& entry : std::filesystem::directory_iterator(input))
      if (entry.is_regular_file()) files.push_back(entry.path().string());
    std::sort(files.begin(), files.end());
    for (size_t g0 = 0; g0 < files.size(); g0 += per_launch) {
      const size_t g1 = std::min(files.size(), g0 + (size_t)per_launch);
      std::cout << "Loading " << (g1 - g0) << " datacubes..." << std::flush;
      std::vector<std::unique_ptr<DataCube>> cubes(g1 - g0);
      std::vector<std::string> errors(g1 - g0);
      std::atomic<size_t> next{0};
      auto load = [&]() {
        for (size_t i; (i = next.fetch_add(1)) < cubes.size();) {
          try {
            auto cube = std::make_unique<DataCube>();
            cube->Load(files[g0 + i], false);
            cubes[i] = std::move(cube);
          } catch (const std::exception& e) {
            errors[i] = e.what();
          }
        }
      };
      const unsigned nt = std::max(1u, std::min<unsigned>(std::thread::hardware_concurrency(), (unsigned)cubes.size()));
      std::vector<std::thread> pool;
      for (unsigned t = 1; t < nt; ++t) pool.emplace_back(load);
      load();
      for (auto& t : pool) t.join();
      for (size_t i = 0; i < cubes.size(); ++i)
        if (!errors[i].empty()) throw std::invalid_argument(files[g0 + i] + ": " + errors[i]);
      std::cout << "Datacubes loaded.\nRendering..." << std::flush;
      std::vector<std::unique_ptr<Camera>> cams;
      std::vector<Camera*> ptrs;
      for (auto& cube : cubes) {
        cube->SetTrilinear(interpolate);
        cube->SetLayout(layout);
        cams.push_back(std::make_unique<Camera>(*cube, pixel_size_deg, plot_fov_h, plot_fov_w));
        cams.back()->SetPosition(pos_x, pos_y, pos_z);
        cams.back()->SetAim(aim, 0.f, 0.f);
        ptrs.push_back(cams.back().get());
      }
      RenderBatch(ptrs);
      std::cout << "Completed rendering.\nExporting..." << std::flush;
      for (size_t i = 0; i < cams.size(); ++i) {
        const std::string name = output + base_name(files[g0 + i]);
        cams[i]->ToFITS(name);
        std::cout << "Exported to " << name << ".fits\n" << std::flush;
      }
    }
  } else {
    std::string base_filename;
    std::unique_ptr<Space> space;
    if (!use_cmem) {
      base_filename = base_name(input);
      std::cout << "Loading datacube...\t" << std::flush;
      auto cube = std::make_unique<DataCube>();
      cube->Init(input, false);
      cube->SetTrilinear(interpolate);
      cube->SetLayout(layout);
      space = std::move(cube);
      std::cout << "Datacube loaded.\nRendering...\t\t" << std::flush;
    } else {
      base_filename = "cmembirp";
      std::cout << "Initialising CMEM...\t" << std::flush;
      auto cmem = std::make_unique<CMEM>();
      // the reference's test is always true, because p has defaults
      // (src/main.cpp:269-281); unset parameters stay 0 ("NULL")
      if (p.size() < 4) throw std::invalid_argument("-p takes four comma-separated values");
      cmem->Init(true, v, b, dipole, p[0], (int)p[1], (int)p[2], (int)p[3], B, alpha, beta, bs, A1, A2, ay_bs, az_bs,
                 density);
      space = std::move(cmem);
      std::cout << "Initialised.\nRendering...\t\t" << std::flush;
    }
    Camera camera(*space, pixel_size_deg, plot_fov_h, plot_fov_w);
    camera.SetPosition(pos_x, pos_y, pos_z);
    camera.SetAim(aim, 0.f, 0.f);
    camera.Render();
    std::cout << "Completed rendering.\nExporting...\t\t" << std::flush;
    camera.ToFITS(output + base_filename);
    std::cout << "Exported to " << output << base_filename << ".fits\n" << std::flush;
  }

  const auto end = high_resolution_clock::now();
  std::cout << "Entire operation took " << duration_cast<milliseconds>(end - start).count() << "ms or "
            << duration_cast<seconds>(end - start).count() << "s" << std::endl;
  return 0;
} catch (const std::exception& e) {
  std::cerr << "birp: " << e.what() << std::endl;
  return 1;
}
