// Instantiations of the walk kernel for DMSIM_GEOM_ELLIPSOID: batched variants (basis phase form).
// Written by gen_instances.py.
#include "walk_kernel.cuh"

namespace dmsim {

WalkFn walk_batch_fn_ellipsoid(int wall, int pm, int width, bool tsm) {
  if (wall == 0 && pm == 1 && width == 2 && tsm == false) return k_walk<DMSIM_GEOM_ELLIPSOID, 0, 1, 2, false, true>;
  if (wall == 0 && pm == 1 && width == 4 && tsm == false) return k_walk<DMSIM_GEOM_ELLIPSOID, 0, 1, 4, false, true>;
  if (wall == 0 && pm == 1 && width == 8 && tsm == false) return k_walk<DMSIM_GEOM_ELLIPSOID, 0, 1, 8, false, true>;
  if (wall == 1 && pm == 1 && width == 2 && tsm == false) return k_walk<DMSIM_GEOM_ELLIPSOID, 1, 1, 2, false, true>;
  if (wall == 1 && pm == 1 && width == 4 && tsm == false) return k_walk<DMSIM_GEOM_ELLIPSOID, 1, 1, 4, false, true>;
  if (wall == 1 && pm == 1 && width == 8 && tsm == false) return k_walk<DMSIM_GEOM_ELLIPSOID, 1, 1, 8, false, true>;
  if (wall == 2 && pm == 1 && width == 2 && tsm == false) return k_walk<DMSIM_GEOM_ELLIPSOID, 2, 1, 2, false, true>;
  if (wall == 2 && pm == 1 && width == 4 && tsm == false) return k_walk<DMSIM_GEOM_ELLIPSOID, 2, 1, 4, false, true>;
  if (wall == 2 && pm == 1 && width == 8 && tsm == false) return k_walk<DMSIM_GEOM_ELLIPSOID, 2, 1, 8, false, true>;
  return nullptr;
}

}  // namespace dmsim
