// Instantiations of the free-flight packed-cylinder walk kernel, wall mode reflect: basis rank x phase per sub-step x block size.
// Written by gen_instances.py.
#include "walk_ff.cuh"

namespace dmsim {

FfFn ff_fn_pcyl_reflect(int rt, bool psub, int nt) {
  if (rt == 2 && psub == false && nt == 1024) return k_pcyl_ff<0, 2, false, 1024>;
  if (rt == 2 && psub == true && nt == 1024) return k_pcyl_ff<0, 2, true, 1024>;
  if (rt == 4 && psub == false && nt == 1024) return k_pcyl_ff<0, 4, false, 1024>;
  if (rt == 4 && psub == true && nt == 1024) return k_pcyl_ff<0, 4, true, 1024>;
  if (rt == 8 && psub == false && nt == 1024) return k_pcyl_ff<0, 8, false, 1024>;
  if (rt == 8 && psub == true && nt == 1024) return k_pcyl_ff<0, 8, true, 1024>;
  return nullptr;
}

}  // namespace dmsim
