// mpm_batch_host.h -- host-side access to a batch for the serving runtime
// (internal to libmpm3d_gpu).
#pragma once

#include <string>
#include <vector>

#include "mpm3d_gpu.h"
#include "mpm_setup.h"

namespace mpm {

// touch every page of a host buffer once (before a device-to-host copy into it)
void prefault_host(void* p, size_t bytes);

struct HostScene;
// stage a scene from a deck on any thread (nullptr + code/err on failure);
// with borrow the deck's particle arrays are used in place, so the scene must
// be committed before the deck may be freed
HostScene* scene_stage(const mpm_deck* d, int steps, std::string& err, int* code, bool borrow = false);
// the scene's set-up (geometry, materials; per-particle inputs are released
// once the scene is resident)
const SceneSetup& scene_setup_of(const HostScene* h);
void scene_free(HostScene* h);
long long scene_np(const HostScene* h);
long long scene_device_bytes(const HostScene* h);
// hand a staged scene to a batch (the batch owns it from then on)
int batch_insert(mpm_batch* b, HostScene* h, int* scene_id);

struct BatchProgress {
  int id;         // scene id
  int istep;      // steps done
  int target;     // steps requested
  long long np;   // particles
  unsigned status;
};

// progress of every resident scene, read from the device in one copy
// (synchronises the batch stream)
int batch_progress(mpm_batch* b, std::vector<BatchProgress>& out);
// restart image of a resident scene (its persistent particle arrays in the
// batch's storage order and its step state) and its restoration into a scene
// of the same deck and layout; the next steps continue bit-identically
int mpm_batch_scene_snapshot(mpm_batch* b, int id, std::vector<unsigned char>& out);
// bytes of that image (-1 for no such scene)
long long mpm_batch_scene_restart_bytes(mpm_batch* b, int id);
int mpm_batch_scene_restore(mpm_batch* b, int id, const unsigned char* in, size_t bytes);
// particles of all resident scenes
long long batch_particles(const mpm_batch* b);
// particle-steps still to run over the resident scenes, and the smallest
// number of steps until one of them finishes (0 when none is resident)
void batch_remaining(mpm_batch* b, const std::vector<BatchProgress>& p, int* min_left);

}  // namespace mpm
