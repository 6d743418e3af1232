// Instantiations of the wide-block packed-cylinder walk kernel, wall mode reflect: basis rank x phase per sub-step x block size.
// Written by gen_instances.py.
#include "walk_wide.cuh"

namespace dmsim {

WideFn wide_fn_pcyl_reflect(int rt, bool psub, int nt) {
  if (rt == 2 && psub == false && nt == 1024) return k_pcyl_wide<0, 2, false, 1024>;
  if (rt == 2 && psub == false && nt == 512) return k_pcyl_wide<0, 2, false, 512>;
  if (rt == 2 && psub == true && nt == 1024) return k_pcyl_wide<0, 2, true, 1024>;
  if (rt == 2 && psub == true && nt == 512) return k_pcyl_wide<0, 2, true, 512>;
  if (rt == 4 && psub == false && nt == 1024) return k_pcyl_wide<0, 4, false, 1024>;
  if (rt == 4 && psub == false && nt == 512) return k_pcyl_wide<0, 4, false, 512>;
  if (rt == 4 && psub == true && nt == 1024) return k_pcyl_wide<0, 4, true, 1024>;
  if (rt == 4 && psub == true && nt == 512) return k_pcyl_wide<0, 4, true, 512>;
  if (rt == 8 && psub == false && nt == 1024) return k_pcyl_wide<0, 8, false, 1024>;
  if (rt == 8 && psub == false && nt == 512) return k_pcyl_wide<0, 8, false, 512>;
  if (rt == 8 && psub == true && nt == 1024) return k_pcyl_wide<0, 8, true, 1024>;
  if (rt == 8 && psub == true && nt == 512) return k_pcyl_wide<0, 8, true, 512>;
  return nullptr;
}

}  // namespace dmsim
