// Drop-in for the reference's Camera (include/Camera.h:20-63): same
// constructor, pose setters, Render, image, ToDat and ToFITS. Render runs the
// fused GB300 kernel and ADDS the result to `image`, as the reference does
// (a second Render doubles the image).
#pragma once
#include <string>
#include <vector>

#include "DataCube.h"

class Camera {
 public:
  Space* dataCube;  // non-owning, as in the reference
  std::vector<std::vector<float>> image;

  Camera(Space& cube, float pixel_size_deg, float plot_fov_h, float plot_fov_w);
  // Explicit image dimensions (the reference derives them as round(fov/pixel)).
  Camera(Space& cube, float plot_fov_h, float plot_fov_w, int nx, int ny);
  ~Camera();

  void SetPosition(float&, float&, float&);
  void SetAim(float, float, float);
  void Render();
  int ToDat(std::string filename);
  int ToFITS(std::string filename);

  // Extensions: sampling along the ray (reference: 200 samples over 44 Re),
  // the march mode (0 PREFIX = reference, 1 CLIP) and lanes per ray.
  void SetSamples(int n_samples, double ray_length = 44.0);
  void SetStep(double step, double ray_length = 44.0);
  void SetMarchMode(int mode);
  void SetSegments(int lanes);
  // Extension: roll about the view axis in degrees, added to the Sun-fixed
  // roll that Orient computes (0, the default, is the reference's pose).
  void SetRoll(double degrees);
  int Width() const { return image_dimension_x; }
  int Height() const { return image_dimension_y; }

 private:
  friend void RenderBatch(const std::vector<Camera*>& cameras);
  birp_camera Describe() const;  // this camera as the C ABI's request
  int image_dimension_x;
  int image_dimension_y;
  float fov_x;
  float fov_y;
  struct {
    float x, y, z;
  } position{0, 0, 0}, aim{0, 0, 0};
  float pixel_size_deg;
  int ray_samples = 200;
  double ray_length = 44.0;
  int march = 0;
  int segments = 0;
  double roll_deg = 0.0;
};

// Renders several cameras (any mix of DataCubes and CMEM) in one batched GPU
// launch (birp_batch_render); each camera's image accumulates its render, as
// Render() does. No reference counterpart: the reference renders one camera
// per call (src/main.cpp:242-264).
void RenderBatch(const std::vector<Camera*>& cameras);
