// Instantiations of the walk kernel for DMSIM_GEOM_PACKED_CYLINDERS.
#include "walk_kernel.cuh"

namespace dmsim {

WalkFn walk_fn_pcyl(int wall, int mt, bool tsm) {
  if (wall == 0 && mt == 4 && tsm == false) return k_walk<DMSIM_GEOM_PACKED_CYLINDERS, 0, 4, false>;
  if (wall == 0 && mt == 4 && tsm == true) return k_walk<DMSIM_GEOM_PACKED_CYLINDERS, 0, 4, true>;
  if (wall == 0 && mt == 16 && tsm == false) return k_walk<DMSIM_GEOM_PACKED_CYLINDERS, 0, 16, false>;
  if (wall == 0 && mt == 16 && tsm == true) return k_walk<DMSIM_GEOM_PACKED_CYLINDERS, 0, 16, true>;
  if (wall == 0 && mt == 32 && tsm == false) return k_walk<DMSIM_GEOM_PACKED_CYLINDERS, 0, 32, false>;
  if (wall == 0 && mt == 32 && tsm == true) return k_walk<DMSIM_GEOM_PACKED_CYLINDERS, 0, 32, true>;
  if (wall == 0 && mt == 64 && tsm == false) return k_walk<DMSIM_GEOM_PACKED_CYLINDERS, 0, 64, false>;
  if (wall == 0 && mt == 64 && tsm == true) return k_walk<DMSIM_GEOM_PACKED_CYLINDERS, 0, 64, true>;
  if (wall == 1 && mt == 4 && tsm == false) return k_walk<DMSIM_GEOM_PACKED_CYLINDERS, 1, 4, false>;
  if (wall == 1 && mt == 4 && tsm == true) return k_walk<DMSIM_GEOM_PACKED_CYLINDERS, 1, 4, true>;
  if (wall == 1 && mt == 16 && tsm == false) return k_walk<DMSIM_GEOM_PACKED_CYLINDERS, 1, 16, false>;
  if (wall == 1 && mt == 16 && tsm == true) return k_walk<DMSIM_GEOM_PACKED_CYLINDERS, 1, 16, true>;
  if (wall == 1 && mt == 32 && tsm == false) return k_walk<DMSIM_GEOM_PACKED_CYLINDERS, 1, 32, false>;
  if (wall == 1 && mt == 32 && tsm == true) return k_walk<DMSIM_GEOM_PACKED_CYLINDERS, 1, 32, true>;
  if (wall == 1 && mt == 64 && tsm == false) return k_walk<DMSIM_GEOM_PACKED_CYLINDERS, 1, 64, false>;
  if (wall == 1 && mt == 64 && tsm == true) return k_walk<DMSIM_GEOM_PACKED_CYLINDERS, 1, 64, true>;
  if (wall == 2 && mt == 4 && tsm == false) return k_walk<DMSIM_GEOM_PACKED_CYLINDERS, 2, 4, false>;
  if (wall == 2 && mt == 4 && tsm == true) return k_walk<DMSIM_GEOM_PACKED_CYLINDERS, 2, 4, true>;
  if (wall == 2 && mt == 16 && tsm == false) return k_walk<DMSIM_GEOM_PACKED_CYLINDERS, 2, 16, false>;
  if (wall == 2 && mt == 16 && tsm == true) return k_walk<DMSIM_GEOM_PACKED_CYLINDERS, 2, 16, true>;
  if (wall == 2 && mt == 32 && tsm == false) return k_walk<DMSIM_GEOM_PACKED_CYLINDERS, 2, 32, false>;
  if (wall == 2 && mt == 32 && tsm == true) return k_walk<DMSIM_GEOM_PACKED_CYLINDERS, 2, 32, true>;
  if (wall == 2 && mt == 64 && tsm == false) return k_walk<DMSIM_GEOM_PACKED_CYLINDERS, 2, 64, false>;
  if (wall == 2 && mt == 64 && tsm == true) return k_walk<DMSIM_GEOM_PACKED_CYLINDERS, 2, 64, true>;
  return nullptr;
}

}  // namespace dmsim
