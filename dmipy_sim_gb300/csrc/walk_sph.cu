// Instantiations of the walk kernel for DMSIM_GEOM_SPHERE.
#include "walk_kernel.cuh"

namespace dmsim {

WalkFn walk_fn_sph(int wall, int mt, bool tsm) {
  if (wall == 0 && mt == 4 && tsm == false) return k_walk<DMSIM_GEOM_SPHERE, 0, 4, false>;
  if (wall == 0 && mt == 16 && tsm == false) return k_walk<DMSIM_GEOM_SPHERE, 0, 16, false>;
  if (wall == 0 && mt == 32 && tsm == false) return k_walk<DMSIM_GEOM_SPHERE, 0, 32, false>;
  if (wall == 0 && mt == 64 && tsm == false) return k_walk<DMSIM_GEOM_SPHERE, 0, 64, false>;
  if (wall == 1 && mt == 4 && tsm == false) return k_walk<DMSIM_GEOM_SPHERE, 1, 4, false>;
  if (wall == 1 && mt == 16 && tsm == false) return k_walk<DMSIM_GEOM_SPHERE, 1, 16, false>;
  if (wall == 1 && mt == 32 && tsm == false) return k_walk<DMSIM_GEOM_SPHERE, 1, 32, false>;
  if (wall == 1 && mt == 64 && tsm == false) return k_walk<DMSIM_GEOM_SPHERE, 1, 64, false>;
  if (wall == 2 && mt == 4 && tsm == false) return k_walk<DMSIM_GEOM_SPHERE, 2, 4, false>;
  if (wall == 2 && mt == 16 && tsm == false) return k_walk<DMSIM_GEOM_SPHERE, 2, 16, false>;
  if (wall == 2 && mt == 32 && tsm == false) return k_walk<DMSIM_GEOM_SPHERE, 2, 32, false>;
  if (wall == 2 && mt == 64 && tsm == false) return k_walk<DMSIM_GEOM_SPHERE, 2, 64, false>;
  return nullptr;
}

}  // namespace dmsim
