// Instantiations of the walk kernel for DMSIM_GEOM_CYLINDER: wall mode x phase form (direct MT / basis RT / vector Bloch) x cell list in shared memory.
// Written by gen_instances.py.
#include "walk_kernel.cuh"

namespace dmsim {

WalkFn walk_fn_cyl(int wall, int pm, int width, bool tsm) {
  if (wall == 0 && pm == 0 && width == 16 && tsm == false) return k_walk<DMSIM_GEOM_CYLINDER, 0, 0, 16, false, false>;
  if (wall == 0 && pm == 0 && width == 32 && tsm == false) return k_walk<DMSIM_GEOM_CYLINDER, 0, 0, 32, false, false>;
  if (wall == 0 && pm == 0 && width == 64 && tsm == false) return k_walk<DMSIM_GEOM_CYLINDER, 0, 0, 64, false, false>;
  if (wall == 0 && pm == 1 && width == 2 && tsm == false) return k_walk<DMSIM_GEOM_CYLINDER, 0, 1, 2, false, false>;
  if (wall == 0 && pm == 1 && width == 4 && tsm == false) return k_walk<DMSIM_GEOM_CYLINDER, 0, 1, 4, false, false>;
  if (wall == 0 && pm == 1 && width == 8 && tsm == false) return k_walk<DMSIM_GEOM_CYLINDER, 0, 1, 8, false, false>;
  if (wall == 0 && pm == 2 && width == 4 && tsm == false) return k_walk<DMSIM_GEOM_CYLINDER, 0, 2, 4, false, false>;
  if (wall == 0 && pm == 2 && width == 16 && tsm == false) return k_walk<DMSIM_GEOM_CYLINDER, 0, 2, 16, false, false>;
  if (wall == 1 && pm == 0 && width == 16 && tsm == false) return k_walk<DMSIM_GEOM_CYLINDER, 1, 0, 16, false, false>;
  if (wall == 1 && pm == 0 && width == 32 && tsm == false) return k_walk<DMSIM_GEOM_CYLINDER, 1, 0, 32, false, false>;
  if (wall == 1 && pm == 0 && width == 64 && tsm == false) return k_walk<DMSIM_GEOM_CYLINDER, 1, 0, 64, false, false>;
  if (wall == 1 && pm == 1 && width == 2 && tsm == false) return k_walk<DMSIM_GEOM_CYLINDER, 1, 1, 2, false, false>;
  if (wall == 1 && pm == 1 && width == 4 && tsm == false) return k_walk<DMSIM_GEOM_CYLINDER, 1, 1, 4, false, false>;
  if (wall == 1 && pm == 1 && width == 8 && tsm == false) return k_walk<DMSIM_GEOM_CYLINDER, 1, 1, 8, false, false>;
  if (wall == 1 && pm == 2 && width == 4 && tsm == false) return k_walk<DMSIM_GEOM_CYLINDER, 1, 2, 4, false, false>;
  if (wall == 1 && pm == 2 && width == 16 && tsm == false) return k_walk<DMSIM_GEOM_CYLINDER, 1, 2, 16, false, false>;
  if (wall == 2 && pm == 0 && width == 16 && tsm == false) return k_walk<DMSIM_GEOM_CYLINDER, 2, 0, 16, false, false>;
  if (wall == 2 && pm == 0 && width == 32 && tsm == false) return k_walk<DMSIM_GEOM_CYLINDER, 2, 0, 32, false, false>;
  if (wall == 2 && pm == 0 && width == 64 && tsm == false) return k_walk<DMSIM_GEOM_CYLINDER, 2, 0, 64, false, false>;
  if (wall == 2 && pm == 1 && width == 2 && tsm == false) return k_walk<DMSIM_GEOM_CYLINDER, 2, 1, 2, false, false>;
  if (wall == 2 && pm == 1 && width == 4 && tsm == false) return k_walk<DMSIM_GEOM_CYLINDER, 2, 1, 4, false, false>;
  if (wall == 2 && pm == 1 && width == 8 && tsm == false) return k_walk<DMSIM_GEOM_CYLINDER, 2, 1, 8, false, false>;
  if (wall == 2 && pm == 2 && width == 4 && tsm == false) return k_walk<DMSIM_GEOM_CYLINDER, 2, 2, 4, false, false>;
  if (wall == 2 && pm == 2 && width == 16 && tsm == false) return k_walk<DMSIM_GEOM_CYLINDER, 2, 2, 16, false, false>;
  return nullptr;
}

}  // namespace dmsim
