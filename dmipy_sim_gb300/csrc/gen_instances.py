"""Writes the walk-kernel instantiation tables (walk_<kind>.cu, walk_batch_<kind>.cu).

Each geometry gets one translation unit of single-instance variants (wall mode x phase form x
cell list in shared memory; the vector-Bloch form for every geometry but the myelinated ones) and, except the myelinated cylinders (whose batch instances run as
plain walks), one of batched variants (basis phase form only), so that the parallel build compiles
them side by side.  Run after changing the variant set.
"""
from pathlib import Path

HERE = Path(__file__).resolve().parent
KINDS = [  # (file stem, enum, wall modes, has a cell list, has batched variants)
    ("free", "DMSIM_GEOM_FREE", [0], False, True),
    ("cyl", "DMSIM_GEOM_CYLINDER", [0, 1, 2], False, True),
    ("sph", "DMSIM_GEOM_SPHERE", [0, 1, 2], False, True),
    ("pcyl", "DMSIM_GEOM_PACKED_CYLINDERS", [0, 1, 2], True, True),
    ("psph", "DMSIM_GEOM_PACKED_SPHERES", [0, 1, 2], True, True),
    ("mesh", "DMSIM_GEOM_MESH", [0, 1, 2], False, True),
    ("myelin", "DMSIM_GEOM_MYELIN", [0, 2], False, False),
    ("pmyelin", "DMSIM_GEOM_PMYELIN", [0, 2], False, False),
    ("box1d", "DMSIM_GEOM_BOX1D", [0, 1], False, True),
    ("slab", "DMSIM_GEOM_SLAB", [0, 1, 2], False, True),
    ("shell", "DMSIM_GEOM_SHELL", [0, 2], False, True),
    ("ellipsoid", "DMSIM_GEOM_ELLIPSOID", [0, 1, 2], False, True),
]
VARIANTS = [(0, 16), (0, 32), (0, 64), (1, 2), (1, 4), (1, 8)]  # (phase form, width)
BLOCH_VARIANTS = [(2, 4), (2, 16)]  # vector Bloch: measurements per pass
NO_BLOCH = {"myelin", "pmyelin"}


def _table(stem, enum, walls, packed, batch):
    tsms = [False, True] if packed else [False]
    fn = f"walk_{'batch_' if batch else ''}fn_{stem}"
    what = ("batched variants (basis phase form)" if batch else
            "wall mode x phase form (direct MT / basis RT / vector Bloch) x cell list in shared "
            "memory")
    lines = [f"// Instantiations of the walk kernel for {enum}: {what}.",
             "// Written by gen_instances.py.",
             '#include "walk_kernel.cuh"', "", "namespace dmsim {", "",
             f"WalkFn {fn}(int wall, int pm, int width, bool tsm) {{"]
    b = "true" if batch else "false"
    variants = VARIANTS + ([] if batch or stem in NO_BLOCH else BLOCH_VARIANTS)
    for wall in walls:
        for pm, width in variants:
            if batch and pm == 0:
                continue
            for tsm in tsms:
                t = "true" if tsm else "false"
                lines.append(f"  if (wall == {wall} && pm == {pm} && width == {width} && tsm == {t}) "
                             f"return k_walk<{enum}, {wall}, {pm}, {width}, {t}, {b}>;")
    lines += ["  return nullptr;", "}", "", "}  // namespace dmsim", ""]
    return "\n".join(lines)


WIDE_WALLS = [(0, "reflect"), (1, "relax"), (2, "permeate")]
WIDE_RANKS = [2, 4, 8]
WIDE_BLOCKS = [1024, 512]


def _wide_table(wall, name):
    """The wide-block packed-cylinder kernels of one wall mode: shape rank x phase per sub-step x
    block size."""
    lines = [f"// Instantiations of the wide-block packed-cylinder walk kernel, wall mode {name}: "
             "basis rank x phase per sub-step x block size.",
             "// Written by gen_instances.py.",
             '#include "walk_wide.cuh"', "", "namespace dmsim {", "",
             f"WideFn wide_fn_pcyl_{name}(int rt, bool psub, int nt) {{"]
    for rt in WIDE_RANKS:
        for psub in ("false", "true"):
            for nt in WIDE_BLOCKS:
                lines.append(f"  if (rt == {rt} && psub == {psub} && nt == {nt}) "
                             f"return k_pcyl_wide<{wall}, {rt}, {psub}, {nt}>;")
    lines += ["  return nullptr;", "}", "", "}  // namespace dmsim", ""]
    return "\n".join(lines)


FF_BLOCKS = [1024]


def _ff_table(wall, name):
    """The free-flight packed-cylinder kernels of one wall mode: shape rank x phase per sub-step
    x block size."""
    lines = [f"// Instantiations of the free-flight packed-cylinder walk kernel, wall mode {name}: "
             "basis rank x phase per sub-step x block size.",
             "// Written by gen_instances.py.",
             '#include "walk_ff.cuh"', "", "namespace dmsim {", "",
             f"FfFn ff_fn_pcyl_{name}(int rt, bool psub, int nt) {{"]
    for rt in WIDE_RANKS:
        for psub in ("false", "true"):
            for nt in FF_BLOCKS:
                lines.append(f"  if (rt == {rt} && psub == {psub} && nt == {nt}) "
                             f"return k_pcyl_ff<{wall}, {rt}, {psub}, {nt}>;")
    lines += ["  return nullptr;", "}", "", "}  // namespace dmsim", ""]
    return "\n".join(lines)


def main():
    for stem, enum, walls, packed, batched in KINDS:
        (HERE / f"walk_{stem}.cu").write_text(_table(stem, enum, walls, packed, False))
        if batched:
            (HERE / f"walk_batch_{stem}.cu").write_text(_table(stem, enum, walls, packed, True))
    for wall, name in WIDE_WALLS:
        (HERE / f"walk_wide_{name}.cu").write_text(_wide_table(wall, name))
        (HERE / f"walk_ff_{name}.cu").write_text(_ff_table(wall, name))


if __name__ == "__main__":
    main()
