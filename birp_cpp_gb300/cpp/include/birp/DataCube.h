// Drop-in for the reference's DataCube (include/DataCube.h:22-49): same public
// fields and methods; the grid is uploaded to GPU memory (FP32, guard-padded,
// per-axis index tables for nonuniform axes) on first use (a render or a
// sample), or by Upload() after the caller edits the public fields.
#pragma once
#include <string>
#include <vector>

#include "Space.h"

class DataCube : public Space {
 public:
  DataCube() = default;
  ~DataCube() override;
  DataCube(const DataCube&) = delete;
  DataCube& operator=(const DataCube&) = delete;

  void Init() override;
  void Init(std::string& filename, bool debug);
  // Builds the cube from axis node coordinates and x-fastest values
  // (values[(k*ny + j)*nx + i] = slices[k][j][i]).
  void Init(const std::vector<double>& xs, const std::vector<double>& ys, const std::vector<double>& zs,
            const std::vector<float>& values);
  // Builds the cube from another Space sampled at the nodes of the given axes
  // (src.GetSample at every node, on `threads` host threads, so the Space's
  // GetSample must then be safe to call concurrently, as the reference's
  // spaces are): a user-defined Space, which has no GPU representation of
  // its own, renders on the GPU as this cube, interpolated between the nodes
  // (a -1 that GetSample returns outside its domain ends a ray there, as the
  // reference's render does). No counterpart in the reference, whose Camera
  // calls GetSample per ray sample.
  void InitFromSpace(Space& src, const std::vector<double>& xs, const std::vector<double>& ys,
                     const std::vector<double>& zs, int threads = 1);
  // Parses an exported MHD .dat file (src/DataCube.cpp:28-138 format).
  void Load(std::string filename, bool debug);
  float GetSample(float x, float y, float z) override;
  // Many samples in one GPU call; -1 outside the box.
  void GetSamples(const float* xyz, int n, float* out);
  void SetTrilinear(bool);
  // Device layout of the GPU copy (BIRP_CUBE_RECORDS, the default;
  // BIRP_CUBE_PAIRS: ~1/4 of the memory, a little slower to render; or
  // BIRP_CUBE_COMPACT: ~1/8 of the memory, slower). No reference counterpart
  // (the reference keeps the cube on the host).
  void SetLayout(int layout);
  // Re-uploads the public fields after they were changed by the caller.
  void Upload();

  std::vector<float> coords_x;
  std::vector<float> coords_y;
  std::vector<float> coords_z;
  struct {
    int x;
    int y;
    int z;
  } size{0, 0, 0};
  float spacing[3] = {0, 0, 0};
  float origin_coords[3] = {0, 0, 0};
  std::vector<std::vector<std::vector<float>>> slices;

  const birp_cube* GpuCube() override;
  bool Trilinear() const override { return trilinear; }

 private:
  void InitMeta();
  bool trilinear = false;
  int layout = BIRP_CUBE_RECORDS;
  birp_cube* gpu = nullptr;
  std::vector<double> ax64[3];  // exact axis coordinates when given as double
};
