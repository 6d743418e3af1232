// Instantiations of the walk kernel for DMSIM_GEOM_CYLINDER.
#include "walk_kernel.cuh"

namespace dmsim {

WalkFn walk_fn_cyl(int wall, int mt, bool tsm) {
  if (wall == 0 && mt == 4 && tsm == false) return k_walk<DMSIM_GEOM_CYLINDER, 0, 4, false>;
  if (wall == 0 && mt == 16 && tsm == false) return k_walk<DMSIM_GEOM_CYLINDER, 0, 16, false>;
  if (wall == 0 && mt == 32 && tsm == false) return k_walk<DMSIM_GEOM_CYLINDER, 0, 32, false>;
  if (wall == 0 && mt == 64 && tsm == false) return k_walk<DMSIM_GEOM_CYLINDER, 0, 64, false>;
  if (wall == 1 && mt == 4 && tsm == false) return k_walk<DMSIM_GEOM_CYLINDER, 1, 4, false>;
  if (wall == 1 && mt == 16 && tsm == false) return k_walk<DMSIM_GEOM_CYLINDER, 1, 16, false>;
  if (wall == 1 && mt == 32 && tsm == false) return k_walk<DMSIM_GEOM_CYLINDER, 1, 32, false>;
  if (wall == 1 && mt == 64 && tsm == false) return k_walk<DMSIM_GEOM_CYLINDER, 1, 64, false>;
  if (wall == 2 && mt == 4 && tsm == false) return k_walk<DMSIM_GEOM_CYLINDER, 2, 4, false>;
  if (wall == 2 && mt == 16 && tsm == false) return k_walk<DMSIM_GEOM_CYLINDER, 2, 16, false>;
  if (wall == 2 && mt == 32 && tsm == false) return k_walk<DMSIM_GEOM_CYLINDER, 2, 32, false>;
  if (wall == 2 && mt == 64 && tsm == false) return k_walk<DMSIM_GEOM_CYLINDER, 2, 64, false>;
  return nullptr;
}

}  // namespace dmsim
