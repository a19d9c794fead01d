// Drop-in for the reference's CMEM (include/Cmem.h:21-97): the 17-argument
// Init with the reference's defaults; coefficients are set up on the host in
// FP64 and the model is evaluated inside the GPU render kernel.
#pragma once
#include <vector>

#include "Space.h"

class CMEM : public Space {
 public:
  CMEM() = default;
  ~CMEM() override;
  CMEM(const CMEM&) = delete;
  CMEM& operator=(const CMEM&) = delete;

  void Init(bool hack, std::vector<int> v_passed = {}, std::vector<int> b_passed = {}, float dipole_passed = 0.f,
            float p0_passed = 0.786300004f, int p1_passed = 1, int p2_passed = 3, int p3_passed = 4,
            float B_passed = 2.f, float alpha_passed = 2.5f, float beta_passed = -1.6f,
            float bs_passed = 12.6400003f, float A1_passed = 7.2e-06f, float A2_passed = 3.5000000000000004e-06f,
            float ay_bs_passed = 0.f, float az_bs_passed = 0.f, float density_passed = 0.f);
  void Init() override;
  float GetSample(float x, float y, float z) override;
  void GetSamples(const float* xyz, int n, float* out);

  const birp_cmem* GpuCmem() override { return gpu; }

 private:
  birp_cmem* gpu = nullptr;
};
