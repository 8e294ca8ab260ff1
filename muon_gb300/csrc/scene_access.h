// Read-only view of a MuonScene's device-side state for entry points that
// live outside render.cc.
#pragma once

#include <cuda_runtime.h>

#include "../../include/muon_gpu.h"
#include "dev_layout.h"
#include "scene_build.h"

namespace muon_gpu {

struct SceneView {
  const DevScene *dev;
  const DevCamera *cam;
  cudaStream_t stream;
  int device;
  int width, height;
  const SceneImage *img;  // host copy of the scene's device arrays
  int64_t num_slots;      // primitive records on the device (dev->prims ...)
};

// Fills `out` from a scene created by muon_gpu_scene_create; false if null.
// The view's host image holds the leaf-order records only after
// SyncSceneImage.
bool GetSceneView(const MuonScene *scene, SceneView *out);
// Copies a device-built scene's records back into its host image (once);
// throws CudaError.
void SyncSceneImage(const MuonScene *scene);

}  // namespace muon_gpu
