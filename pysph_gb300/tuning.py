"""Launch-shape choices for the GPU neighbour structure and pair kernels.

``choose_subdivision`` picks how many internal grid cells span one
reference cell (``cell_size = 2 max h``).  Finer cells cut the candidate
volume a destination must test (27 cells of (2h)^3 at 1, 125 of h^3 at 2,
343 of (2h/3)^3 at 3) at the cost of more, shorter rows.  The default comes
from a per-dimension table measured on GB300 (1 M-particle 3D lattice: 3.18,
2.40 and 2.33 ms per RK2 step at subdivisions 1, 2, 3);
``PYSPH_GB300_SUBDIV`` overrides it.
"""
import os

# neighbour-list skin, as a fraction of the search radius: a full neighbour
# build keeps the sources within (1 + skin) times the radius, and later
# updates only refresh the sorted state while no particle has moved by half
# the skin (PYSPH_GB300_SKIN overrides; 0 rebuilds at every update like the
# reference)
DEFAULT_SKIN = 0.03


# small simulations whose lists go stale within a few steps (the motion of
# a step reaches half the skin): every SKIN_WINDOW steps the skin doubles,
# up to SKIN_MAX, while the window had more than one full build per four
# steps -- longer-lived lists let a recorded step replay as one graph, and
# below GRAPH_MAX_PARTICLES the launches, not the longer lists, bound a step
SKIN_WINDOW = 16
SKIN_MAX = 0.24



def list_skin():
    env = os.environ.get("PYSPH_GB300_SKIN")
    if env is not None:
        v = float(env)
        if not 0.0 <= v <= 0.5:
            raise ValueError("PYSPH_GB300_SKIN must be in [0, 0.5]")
        return v
    return DEFAULT_SKIN


def skin_growth(nparticles):
    """(window, builds above which the skin grows, factor, ceiling) of the
    integrators' skin adaptation, or None: PYSPH_GB300_SKIN set, or a
    simulation of GRAPH_MAX_PARTICLES or more, whose step time is flat
    around the default (1 M particles of the jittered lattice, 300 RK2
    steps: 1.118 / 1.098 / 1.111 / 1.104 / 1.113 / 1.124 ms per step at
    skins 0.015 / 0.02 / 0.025 / 0.03 / 0.04 / 0.05; 16.8 M: 18.25 ms at
    0.03 against 18.33 ms with the skin grown to 0.0675 whenever a window
    of 32 steps had more than 5 full builds)."""
    if os.environ.get("PYSPH_GB300_SKIN") is not None or nparticles >= GRAPH_MAX_PARTICLES:
        return None
    return SKIN_WINDOW, SKIN_WINDOW // 4, 2.0, SKIN_MAX


def brick_passes():
    """Whether the pair passes that qualify (one source of uniform h, no
    periodic axis or variable-h relation) run the brick-staged kernels, which
    stage each brick of cells' neighbour records in shared memory
    (PYSPH_GB300_BRICKS=0 selects the list-streaming kernels everywhere)."""
    env = os.environ.get("PYSPH_GB300_BRICKS")
    if env is not None:
        if env not in ("0", "1"):
            raise ValueError("PYSPH_GB300_BRICKS must be 0 or 1")
        return env == "1"
    return True


# below this many particles a step is shorter than the host's calls for it,
# and replaying it as one graph pays; above it the step is device-bound (1 M
# particles: 1.222 ms per replayed step against 1.214 call by call) and the
# calls' deferred checks keep host transfers overlapped with the steps
GRAPH_MAX_PARTICLES = 500_000


def step_graphs(nparticles=0):
    """Whether integrators record their step once and replay it as one CUDA
    graph per step: PYSPH_GB300_GRAPHS=1 always, 0 never, unset (auto) for
    simulations of fewer than GRAPH_MAX_PARTICLES particles."""
    env = os.environ.get("PYSPH_GB300_GRAPHS")
    if env is not None:
        if env not in ("0", "1"):
            raise ValueError("PYSPH_GB300_GRAPHS must be 0 or 1")
        return env == "1"
    return nparticles < GRAPH_MAX_PARTICLES


# measured defaults: (dimensions with extent) -> subdivision; with the
# brick-staged passes (one uniform h) the 3D optimum is 2 (1 M-particle
# lattice, RK2 step: 1.05 ms at subdivision 2 with 6 x 5 x 5-cell bricks
# against 1.10 ms at 3 with 8^3-cell bricks), for the list-streaming
# passes 3
DEFAULT_SUBDIVISION = {1: 1, 2: 2, 3: 3}
DEFAULT_SUBDIVISION_BRICKS = {1: 1, 2: 2, 3: 2}
# neighbour-list entries hold the source slot in 32 - code bits (three
# fields of 2 bits at subdivision 1, of 3 bits at 3; at subdivision 2 three
# 3-bit fields up to 2^23 particles, above that the offset in base 5 in 7
# bits): at most 2^26 source particles at subdivision 1, 2^25 at 2, 2^23 at 3
MAX_PARTICLES = {1: 1 << 26, 2: 1 << 25, 3: 1 << 23}


def choose_subdivision(cell_manager):
    env = os.environ.get("PYSPH_GB300_SUBDIV")
    if env:
        v = int(env)
        if v not in (1, 2, 3):
            raise ValueError("PYSPH_GB300_SUBDIV must be 1, 2 or 3")
        return v
    dims = 1
    for pa in cell_manager.arrays_to_bin:
        if pa.get_number_of_particles() == 0:
            continue
        for k, c in ((2, "y"), (3, "z")):
            t = pa.get_device(c)
            if t.numel() and float(t.max() - t.min()) > 0:
                dims = max(dims, k)
    table = DEFAULT_SUBDIVISION
    if brick_passes():
        hs = [pa.get_device("h") for pa in cell_manager.arrays_to_bin
              if pa.get_number_of_particles() > 0]
        if hs and all(float(h.max()) == float(h.min()) for h in hs) and \
                len({float(h[0]) for h in hs}) == 1:
            table = DEFAULT_SUBDIVISION_BRICKS
    sub = table[dims]
    nmax = max((pa.get_number_of_particles() for pa in cell_manager.arrays_to_bin), default=0)
    while sub > 1 and nmax >= MAX_PARTICLES[sub]:
        sub -= 1
    return sub


def time_batch_steps(batch, steps):
    """Device time (ms) of ``steps`` batch steps, from CUDA events recorded
    on the batch's stream."""
    import torch
    st = batch.stream()
    batch.step(1)                       # captures the graph (not timed)
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record(st)
    batch.step(steps, check=False)
    b.record(st)
    b.synchronize()
    batch.check()
    return a.elapsed_time(b)


def autotune_batch(instances, candidates=(1, 2, 3), steps=5, count_bins=3, dx_bins=2,
                   **recipe):
    """Choose each instance's cell subdivision by timing.

    The instances are binned by particle count (``count_bins`` bins of
    equal membership over the sorted counts) and, within a count bin, by
    resolution (``dx_bins`` bins over their smoothing lengths).  Every bin's
    instances are timed as a batch of their own at each candidate
    subdivision (``steps`` graph steps after the capture), and every
    instance gets its bin's fastest.  The whole batch is timed too, at each
    candidate for all instances and with the per-bin choices; the fastest
    of these is returned.  Returns ``(subdivs, report)``: one subdivision
    per instance and the timings (ms per step)."""
    from .batch import SimulationBatch
    import copy
    import numpy as np
    n = np.array([len(p["x"]) for p in instances])
    h = np.array([float(np.max(p["h"])) for p in instances])
    order = np.argsort(n, kind="stable")
    bins = []
    for cb in np.array_split(order, max(1, min(count_bins, len(order)))):
        if len(cb) == 0:
            continue
        hb = cb[np.argsort(h[cb], kind="stable")]
        for db in np.array_split(hb, max(1, min(dx_bins, len(hb)))):
            if len(db):
                bins.append(sorted(int(i) for i in db))

    def timed(insts, sub):
        b = SimulationBatch(copy.deepcopy(insts), subdiv=sub, **recipe)
        ms = time_batch_steps(b, steps) / steps
        del b
        return ms

    choice = [candidates[0]] * len(instances)
    per_bin = []
    for members in bins:
        sub_insts = [instances[i] for i in members]
        t = {sub: timed(sub_insts, sub) for sub in candidates}
        best = min(t, key=t.get)
        for i in members:
            choice[i] = best
        per_bin.append({"instances": len(members), "particles": int(n[members].sum()),
                        "ms_per_step": t, "subdiv": best})
    whole = {str(sub): timed(instances, sub) for sub in candidates}
    whole["per_instance"] = timed(instances, choice)
    best_uniform = min(candidates, key=lambda c: whole[str(c)])
    if whole[str(best_uniform)] < whole["per_instance"]:
        choice = [best_uniform] * len(instances)
    report = {"bins": per_bin, "whole_batch_ms_per_step": whole,
              "chosen": "per_instance" if len(set(choice)) > 1 or
                        whole["per_instance"] <= whole[str(best_uniform)] else str(best_uniform)}
    return choice, report
