// mpm_setup.h -- a scene's set-up derived from a parsed deck (host side).
#pragma once

#include <string>
#include <vector>

#include "mpm_deck.h"
#include "mpm_gpu_internal.cuh"

namespace mpm {

struct SceneSetup {
  Geometry g;
  std::vector<DevMaterial> mats;
  std::vector<DevBody> bodies;  // mat = 0-based index into mats
  std::vector<double> vol, sig_y, ie, cp, lt;  // per particle (Initial)
  std::vector<uint8_t> fix, bd;                // per node
  std::string err;
};

// Initial + SetGridData of a deck; returns an mpm_status. particle_fields:
// also fill the per-particle vol / sig_y / ie / cp / lt (the batched engine
// derives them on the device instead).
int scene_setup(const mpm_deck* d, SceneSetup& out, bool particle_fields = true);
// SetDT: the first time step of a material set.
double set_dt(const std::vector<DevMaterial>& mats, double dcell, double dtscale);

}  // namespace mpm
