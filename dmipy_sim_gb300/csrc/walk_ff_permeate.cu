// Instantiations of the free-flight packed-cylinder walk kernel, wall mode permeate: basis rank x phase per sub-step x block size.
// Written by gen_instances.py.
#include "walk_ff.cuh"

namespace dmsim {

FfFn ff_fn_pcyl_permeate(int rt, bool psub, int nt) {
  if (rt == 2 && psub == false && nt == 1024) return k_pcyl_ff<2, 2, false, 1024>;
  if (rt == 2 && psub == true && nt == 1024) return k_pcyl_ff<2, 2, true, 1024>;
  if (rt == 4 && psub == false && nt == 1024) return k_pcyl_ff<2, 4, false, 1024>;
  if (rt == 4 && psub == true && nt == 1024) return k_pcyl_ff<2, 4, true, 1024>;
  if (rt == 8 && psub == false && nt == 1024) return k_pcyl_ff<2, 8, false, 1024>;
  if (rt == 8 && psub == true && nt == 1024) return k_pcyl_ff<2, 8, true, 1024>;
  return nullptr;
}

}  // namespace dmsim
