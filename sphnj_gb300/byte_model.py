"""Algorithmic (compulsory) HBM bytes of each pass of the particle step.

Each pass reads each particle's inputs once and writes its outputs once;
neighbour re-reads are not counted.  Sizes are those of the plain form
(fluid FP32, solid FP64, 1-byte enums).  Per particle:

  pass                      bytes   made of
  bin (cell ids)            12      read position 8, write cell id 4
  rebuild (fluid lists)     15      cell id 4 + list entry r 4 / w 4 + ranges ~3
  sort (every 50 steps)     2       amortised
  fluid_pair                67      read pos 8, vel 8, rho 4, p 4, phase 1, cell 4 = 29 (26 +
                                    cell id); write drho 4, du_dt 8, near 1, color 4,
                                    gradient 8, du_dx 16 = 41
  fluid_update              57      read pos 8, vel 8, du_dt 8, rho 4, drho 4, phase 1 = 33;
                                    write pos 8, vel 8, rho 4, p 4 = 24
  shift_pass                54      one shifting pass, gradient and update in one sweep:
                                    read pos 8, color 4, near 1, phase 1, du_dx 16, vel 8 = 38;
                                    write pos 8 (the other buffer), vel 8 = 16
  shift_last                9       the step's last pass also writes the gradient 8 and the
                                    boundary type 1 (earlier passes' values are never read)
  shift_copy_back           16      read pos 8, write pos 8 (odd S only)
  virt_data (per virtual)   34      read pos 8, normal 8, phase 1, boundary 1, cell 4;
                                    write vel 8, p 4, rho 4, phase 1 (~34 with the cell id)
  solid per fluid step      48      bin 20 + coupling 28
  solid per sub-step        440     deformation ~178 + force ~181 + update ~81

B_step = N_f (153 + 54 S + 9 [S > 0] + 16 [S odd]) + N_v 46 + N_s (48 + 440 k)
(S shifting passes, k solid sub-steps)
"""
from __future__ import annotations

PER_PARTICLE = {
    "bin": 12,
    "bin_solid": 20,  # FP64 position 16 + cell id 4
    "rebuild": 15,
    "sort": 2 * 50,  # per sort call (the amortised 2 B/step of the model, over 50 steps)
    "fluid_pair": 67,
    "fluid_update": 57,
    "shift_pass": 54,
    "shift_last": 9,
    "shift_copy_back": 16,
    "virt_data": 34,
    "solid_couple": 28,
    "solid_deformation": 178,
    "solid_force": 181,
    "solid_update": 81,
}

# which particle count a stage's bytes scale with
STAGE_KIND = {
    "bin": "all", "bin_solid": "solid", "rebuild": "fluid", "sort": "fluid", "fluid_pair": "fluid", "fluid_update": "fluid",
    "shift_pass": "fluid", "shift_last": "fluid", "shift_copy_back": "fluid", "virt_data": "virt", "solid_couple": "solid",
    "solid_deformation": "solid", "solid_force": "solid", "solid_update": "solid", "capacity": "none",
}


# The mixed-precision form's own field sizes, for the passes that differ
# (the rest are as above):
#   bin             20   read cell 4 + offset 8, write cell 4 + offset 8 when a particle
#                        changes cell (counted always: 12 + 8)
#   fluid_pair      71   the pair pass's 67 + 4: the home position is a cell id 4 and an
#                        offset 8
#   fluid_update    89   57 + offset and velocity compensations read and written 32
#   shift_pass      42   read cell 4 + offset 8, color 4, near 1, phase 1, offset
#                        compensation 8 = 26; write offset 8, compensation 8 = 16.  A
#                        listed particle's velocity correction is linear in the shift with
#                        a du_dx no pass changes, so it is applied once, in the last pass
#   shift_last      73   gradient 8 and boundary type 1 written; du_dx 16, velocity and its
#                        compensation 16, offset and compensation before the first pass 16
#                        read; velocity and compensation written 16
#   solid passes         FP32 state: deformation 8 + 8 + 8 + 8 read (reference cell, offset,
#                        displacement of i; neighbours counted once) + writes F, P, L 96 and
#                        P L, F L 32 = 160; force 8 + 8 + 8 + 16 + 16 + 4 + 1 read, 16 write = 77;
#                        update 8 + 8 + 8 + 8 + 8 + 1 + 8 read (+ reference cell / offset 16 for the
#                        current offset), 8 x 5 write = 105
PER_PARTICLE_MIXED = dict(PER_PARTICLE, bin=20, bin_solid=20, fluid_pair=71, fluid_update=89, shift_pass=42, shift_last=73,
                          solid_deformation=160, solid_force=77, solid_update=105)


def bytes_per_launch(stage: str, nf: int, ns: int, nv: int, mixed: bool = False, shifts: int = 0) -> float:
    """Compulsory bytes of one launch of a stage; for the shifting passes the
    average launch of a step of `shifts` passes (the last one writes more)."""
    t = PER_PARTICLE_MIXED if mixed else PER_PARTICLE
    kind = STAGE_KIND.get(stage, "none")
    n = {"all": nf + ns + nv, "fluid": nf, "solid": ns, "virt": nv, "none": 0}[kind]
    b = float(t.get(stage, 0))
    if stage == "shift_pass" and shifts > 0:
        b += t["shift_last"] / shifts
    return b * n


def step_bytes(nf: int, ns: int, nv: int, shifts: int, substeps: int, mixed: bool = False) -> float:
    """Compulsory bytes of one step of one scene in either form, from the
    per-pass table of that form: every particle binned, the fluid's list
    rebuild (the sort amortised), pair pass, update and shifting passes, the
    virtual particles' data, and for solids the coupling pass (with fluid) and
    k sub-steps of deformation, force and update."""
    t = PER_PARTICLE_MIXED if mixed else PER_PARTICLE
    b = (nf + nv) * t["bin"] + ns * t["bin_solid"]
    if nf:
        b += nf * (t["rebuild"] + t["sort"] / 50 + t["fluid_pair"] + t["fluid_update"] + shifts * t["shift_pass"]
                   + (shifts > 0) * t["shift_last"] + (shifts & 1) * t["shift_copy_back"])
    b += nv * t["virt_data"]
    if ns:
        b += ns * ((t["solid_couple"] if nf else 0) + substeps * (t["solid_deformation"] + t["solid_force"]
                                                                   + t["solid_update"]))
    return float(b)


def bytes_per_step(nf: int, ns: int, nv: int, shifts: int, substeps: int) -> float:
    """The plain form's step_bytes (the closed formula of the table above)."""
    return step_bytes(nf, ns, nv, shifts, substeps, mixed=False)


# DRAM traffic (dram__bytes_read.sum + dram__bytes_write.sum) per fluid
# particle of one launch of the tiled neighbour sweeps, from one ncu capture of
# the 2,083,750-particle gas-liquid dam break per form (tiles of 16 cells,
# stored neighbour lists, 128-thread blocks; the shifting launch is a pass
# before the step's last); it grows in proportion to the particle count (same
# tile shape, same list length per particle).  Well above the compulsory
# bytes above: the pair pass writes the per-step neighbour lists and every
# shifting pass reads them back (about 96 B per particle).  The captures
# predate the lists of the particles next to a wall, whose tiles' shifting
# passes also stage their virtual strips (7% of that scene's tiles).
MEASURED_TRAFFIC_PER_PARTICLE = {
    "fluid_pair": 148.9,
    "shift_pass": 154.1,
}
MEASURED_TRAFFIC_PER_PARTICLE_MIXED = {
    "fluid_pair": 148.1,
    "shift_pass": 130.6,
}
# issue slots busy (smsp__issue_active, % of peak) of the same captures: the
# neighbour sweeps are bound by instruction issue and latency, not by DRAM
ISSUE_ACTIVE = {"fluid_pair": 0.749, "shift_pass": 0.762}
ISSUE_ACTIVE_MIXED = {"fluid_pair": 0.660, "shift_pass": 0.665}


def measured_traffic_per_launch(stage: str, nf: int, mixed: bool = False) -> float | None:
    b = (MEASURED_TRAFFIC_PER_PARTICLE_MIXED if mixed else MEASURED_TRAFFIC_PER_PARTICLE).get(stage)
    return None if b is None else float(b * nf)
