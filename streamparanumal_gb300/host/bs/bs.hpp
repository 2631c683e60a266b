// Shared declarations of the BS0-BS8 drivers.
#pragma once

#include "mesh.hpp"

namespace libp {

void bs0Settings(settings_t& s);
void bsVecSettings(settings_t& s);
void bsOgsSettings(settings_t& s);
// Applies the per-degree kernel choice of the tuning table before the mesh's plan is
// built (-t/--tuning FILE; default the package's table, NONE to keep the defaults).
void bsOgsApplyTuning(settings_t& s);
void bs0Run(platform_t& platform, settings_t& settings);
void bsVecRun(int which, platform_t& platform, settings_t& settings);
void bsOgsRun(int which, platform_t& platform, settings_t& settings, mesh_t& mesh);

}  // namespace libp
