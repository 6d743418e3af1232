"""dmipy_sim_gb300 — GB300-native Monte-Carlo diffusion-MRI forward walk.

Drop-in for dmipy-sim's ``simulate`` / ``simulate_cpmg`` / ``simulate_trajectories`` /
``replay`` path: the same Waveform and geometry objects and signatures, with the per-walker step
loop executed by hand-written sm_103a CUDA kernels (``libdmsim.so``, C ABI in include/dmsim.h).
"""
from .constants import GAMMA, DEFAULT_SLEW_RATE
from .waveforms import (Waveform, pgse, pgste, ogse, cpmg, calc_b, calc_btensor, set_b,
                        rotate_waveform, tile_waveform, trapezoidal_ogse, b_trapezoidal_ogse,
                        btensor_invariants, ste, pte)
from .geometries import (Geometry, FreeDiffusion, Cylinder, Sphere, MyelinatedCylinder,
                         PackedMyelinatedCylinders, pack_myelinated_cylinders, Box1D,
                         PermeableSlab1D, PermeableShell, Ellipsoid, pack_cylinders,
                         PackedCylinders, pack_spheres, PackedSpheres, lattice_cylinders)
from .core import (simulate, simulate_mixture, simulate_cpmg, simulate_trajectories, run_walk,
                   WalkResult,
                   permeable_sub_steps, surface_sub_steps, collision_sub_steps, replay_sub_steps,
                   fused_sub_steps, mt_sub_steps)
from . import trajectories
from .trajectories import (replay_bloch, replay_bloch_jax, unwrap_periodic, pathway_sign_se,
                           finite_180_longitudinal_dwell, pre_pulse_gradient_phase)
from .mesh import Mesh, load_ply, icosphere, random_ellipsoid_cells, mesh_contains
from .batched import Instance, Tuning, PreparedBatch, simulate_batch
from .autotune import autotune
# as in the reference, the trajectory replay is trajectories.replay and the name ``replay`` is
# the replay-pack module
from . import compression, bank, replay
from .replay import ReplayPack, read_rpk, write_rpk, compile_scheme, replay_signal
from .bank import build_replay_pack, build_to_floor
from . import bloch, mt, mt_walk, pulse_sequence, rf, susceptibility
from .susceptibility import SusceptibilitySources, MyelinSusceptibility, GridSusceptibility
from .rf import B1Pulse, bloch_simulate, slice_profile
from .mt_walk import simulate_mt_trajectories
from .bloch import simulate_bloch
from .pulse_sequence import (BlochSequence, gradient_echo, spin_echo, prepend_mt_prep,
                             run_bloch_sequence, emergent_z_spectrum)

__all__ = [
    "GAMMA", "DEFAULT_SLEW_RATE", "Waveform", "pgse", "pgste", "ogse", "cpmg", "calc_b",
    "calc_btensor", "set_b", "rotate_waveform", "tile_waveform", "trapezoidal_ogse",
    "b_trapezoidal_ogse", "btensor_invariants", "ste", "pte", "Geometry", "FreeDiffusion",
    "Cylinder", "Sphere", "MyelinatedCylinder", "PackedMyelinatedCylinders",
    "pack_myelinated_cylinders", "Box1D", "PermeableSlab1D", "PermeableShell", "Ellipsoid",
    "pack_cylinders", "PackedCylinders", "pack_spheres", "PackedSpheres", "lattice_cylinders",
    "simulate", "simulate_mixture", "simulate_cpmg", "simulate_trajectories", "trajectories", "replay_bloch",
    "replay_bloch_jax", "unwrap_periodic", "pathway_sign_se", "finite_180_longitudinal_dwell",
    "pre_pulse_gradient_phase", "run_walk", "WalkResult",
    "permeable_sub_steps", "surface_sub_steps", "collision_sub_steps", "replay_sub_steps",
    "fused_sub_steps", "mt_sub_steps", "Mesh", "load_ply", "icosphere", "random_ellipsoid_cells", "mesh_contains",
    "Instance", "Tuning", "PreparedBatch", "simulate_batch", "autotune", "compression", "bank", "replay",
    "ReplayPack", "read_rpk", "write_rpk", "compile_scheme", "replay_signal", "build_replay_pack",
    "build_to_floor", "bloch", "mt", "mt_walk", "rf", "susceptibility", "SusceptibilitySources",
    "MyelinSusceptibility", "GridSusceptibility", "B1Pulse", "bloch_simulate", "slice_profile", "simulate_mt_trajectories", "pulse_sequence", "simulate_bloch",
    "BlochSequence", "gradient_echo", "spin_echo", "prepend_mt_prep", "run_bloch_sequence",
    "emergent_z_spectrum",
]
