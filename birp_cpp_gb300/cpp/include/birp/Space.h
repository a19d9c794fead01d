// Drop-in for the reference's Space interface (include/Space.h:18-23): the
// abstract emissivity field a Camera samples. The two pure virtuals keep the
// reference's signatures; the GPU handles let Camera::Render launch the
// fused GB300 kernels instead of calling GetSample per sample.
#pragma once

#include "birp_gb300.h"  // the C ABI the classes call (the include/ directory on the include path)

class Space {
 public:
  virtual ~Space() = default;
  virtual void Init() = 0;
  virtual float GetSample(float x, float y, float z) = 0;
  // GPU representation (exactly one is non-null for the built-in spaces). A
  // user-defined Space without one cannot be rendered directly (there is no
  // CPU path); DataCube::InitFromSpace samples it onto a grid that renders.
  virtual const birp_cube* GpuCube() { return nullptr; }
  virtual const birp_cmem* GpuCmem() { return nullptr; }
  virtual bool Trilinear() const { return false; }
};
