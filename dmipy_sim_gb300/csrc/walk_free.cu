// Instantiations of the walk kernel for DMSIM_GEOM_FREE.
#include "walk_kernel.cuh"

namespace dmsim {

WalkFn walk_fn_free(int wall, int mt, bool tsm) {
  if (wall == 0 && mt == 4 && tsm == false) return k_walk<DMSIM_GEOM_FREE, 0, 4, false>;
  if (wall == 0 && mt == 16 && tsm == false) return k_walk<DMSIM_GEOM_FREE, 0, 16, false>;
  if (wall == 0 && mt == 32 && tsm == false) return k_walk<DMSIM_GEOM_FREE, 0, 32, false>;
  if (wall == 0 && mt == 64 && tsm == false) return k_walk<DMSIM_GEOM_FREE, 0, 64, false>;
  return nullptr;
}

}  // namespace dmsim
