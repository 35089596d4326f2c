"""Checkpoint / resume of device state (the reference's CheckpointSession).

Reference: src/infrastructure/checkpointing.jl -- init_checkpoint(file, state) (:70),
checkpoint!(ckpt; kwargs...) with an atomic tmp + mv write (:48-56),
restore_checkpoint(path) (:95-100), finalize!(ckpt) (:108-111).

Device objects (lattices, algorithms with their counter-based streams, parallel
tempering ladders, flat-histogram ensembles) are exported to host arrays; because
every random number is a function of (seed, stream, counter), a restored run continues
bit for bit where the checkpointed one would have.
"""
import io
import os
import pickle

import numpy as np

from . import (Philox, Metropolis, Glauber, HeatBath, BoltzmannEnsemble, IsingDevice, BlumeCapelDevice, Ising,
               BlumeCapel, default_context, ArgumentError)
from . import flathist as F
from . import pt as PT

__all__ = ["CheckpointSession", "init_checkpoint", "checkpoint_", "restore_checkpoint", "finalize_", "export_state",
           "import_state"]


# ------------------------------------------------------------ export / import --
def export_state(obj):
    """Host-side description of a device object (nested dicts of numbers and arrays)."""
    if isinstance(obj, (IsingDevice, BlumeCapelDevice)):
        return {"kind": "lattice", "model": "bc" if isinstance(obj, BlumeCapelDevice) else "ising",
                "dims": list(obj.dims), "J": obj.J, "D": obj.D, "h": obj.h, "layout": obj.layout,
                "uniforms": obj.uniforms, "spins": obj.spins}
    from .graph import GraphDevice
    if isinstance(obj, GraphDevice):
        return {"kind": "graph", "model": obj.MODEL, "rowptr": obj.rowptr, "col": obj.col, "coupling": obj.coupling,
                "J": obj.J, "D": obj.D, "field": obj.field, "h": obj.h, "spins": obj.spins}
    if isinstance(obj, Philox):
        return {"kind": "rng", "seed": obj.seed, "stream": obj.stream, "counter": obj.counter}
    if isinstance(obj, (Metropolis, Glauber)):
        return {"kind": type(obj).__name__, "beta": obj.beta, "rng": export_state(obj.rng), "steps": obj.steps,
                "accepted": obj.accepted}
    if isinstance(obj, HeatBath):
        return {"kind": "HeatBath", "beta": obj.beta, "rng": export_state(obj.rng), "steps": obj.steps,
                "flips": obj.flips}
    if isinstance(obj, (F.MulticanonicalEnsemble, F.WangLandauEnsemble)):
        import ctypes as C
        from . import _lib as L, _check
        vis = np.empty(obj.bins.nbins, np.uint8)
        _check(L.load().mcx_flathist_get_visited(obj.handle, vis.ctypes.data, vis.size))
        d = {"kind": type(obj).__name__, "bins": (obj.bins.start, obj.bins.step, obj.bins.nbins),
             "logweight": obj.logweight, "histogram": obj.histogram, "visited": vis}
        if isinstance(obj, F.WangLandauEnsemble):
            d["logf"] = obj.logf
        return d
    if isinstance(obj, F._FlatAlg):
        return {"kind": "FlatAlg", "ensemble": export_state(obj.ensemble), "rng": export_state(obj.rng),
                "steps": obj.steps, "accepted": obj.accepted}
    if isinstance(obj, PT.ParallelTempering):
        s, a = obj.counters()
        return {"kind": "ParallelTempering", "dim": obj.dim, "J": obj.J, "h": obj.h,
                "ladders": [(L, list(b)) for L, b in zip(obj.sides, obj.ladder_betas)],
                "rng": export_state(obj.rng), "positions": obj.positions, "stage": obj.stage,
                "steps": s, "accepted": a, "spins": [obj.spins(r) for r in range(obj.nrep)]}
    if isinstance(obj, (list, tuple)):
        return {"kind": "list", "items": [export_state(x) for x in obj]}
    if isinstance(obj, (int, float, str, bool, np.ndarray)) or obj is None:
        return {"kind": "value", "value": obj}
    raise ArgumentError("cannot checkpoint %s" % type(obj).__name__)


def import_state(d, ctx=None):
    """Rebuild a device object from export_state's description."""
    import ctypes as C
    from . import _lib as L, _check
    ctx = ctx or default_context()
    k = d["kind"]
    if k == "value":
        return d["value"]
    if k == "list":
        return [import_state(x, ctx) for x in d["items"]]
    if k == "rng":
        return Philox(d["seed"], d["stream"], d["counter"])
    if k == "lattice":
        if d["model"] == "bc":
            s = BlumeCapel(d["dims"], J=d["J"], D=d["D"], h=d["h"], ctx=ctx)
        else:
            s = Ising(d["dims"], J=d["J"], h=d["h"], layout=d["layout"], ctx=ctx)
        if d.get("uniforms", "site") != "site":
            s.set_uniforms(d["uniforms"])
        s.spins = d["spins"]
        return s
    if k == "graph":
        from .graph import IsingGraphDevice, BlumeCapelGraphDevice
        J = 1.0 if d["J"] is None else d["J"]
        h = d["field"] if d["field"] is not None else d["h"]
        if d.get("model", "Ising") == "BlumeCapel":
            s = BlumeCapelGraphDevice(d["rowptr"], d["col"], d["coupling"], J=J, D=d["D"], h=h, ctx=ctx)
        else:
            s = IsingGraphDevice(d["rowptr"], d["col"], d["coupling"], J=J, h=h, ctx=ctx)
        s.spins = d["spins"]
        return s
    if k in ("Metropolis", "Glauber"):
        a = (Metropolis if k == "Metropolis" else Glauber)(import_state(d["rng"]), beta=d["beta"])
        a.steps, a.accepted = d["steps"], d["accepted"]
        return a
    if k == "HeatBath":
        a = HeatBath(import_state(d["rng"]), beta=d["beta"])
        a.steps, a.flips = d["steps"], d["flips"]
        return a
    if k in ("MulticanonicalEnsemble", "WangLandauEnsemble"):
        if k == "WangLandauEnsemble":
            e = F.WangLandauEnsemble(tuple(d["bins"]), logf=d["logf"], ctx=ctx)
        else:
            e = F.MulticanonicalEnsemble(tuple(d["bins"]), ctx=ctx)
        e.logweight = d["logweight"]
        e.histogram = d["histogram"]
        vis = np.ascontiguousarray(d["visited"], np.uint8)
        _check(L.load().mcx_flathist_set_visited(e.handle, vis.ctypes.data, vis.size))
        return e
    if k == "FlatAlg":
        a = F._FlatAlg(import_state(d["rng"]), import_state(d["ensemble"], ctx))
        a.steps, a.accepted = d["steps"], d["accepted"]
        return a
    if k == "ParallelTempering":
        p = PT.ParallelTempering([(L_, b) for L_, b in d["ladders"]], dim=d["dim"], J=d["J"], h=d["h"], ctx=ctx)
        p.rng = import_state(d["rng"])
        for r, sp in enumerate(d["spins"]):
            p.set_spins_(r, sp)
        pos = np.ascontiguousarray(d["positions"], np.int32)
        _check(L.load().mcx_pt_set_indices(p.handle, pos.ctypes.data, int(d["stage"])))
        st = np.ascontiguousarray(d["steps"], np.uint64)
        ac = np.ascontiguousarray(d["accepted"], np.uint64)
        _check(L.load().mcx_pt_set_exchange_counters(p.handle, st.ctypes.data, ac.ctypes.data))
        return p
    raise ArgumentError("unknown checkpoint entry %s" % k)


# ------------------------------------------------------------------ sessions --
class CheckpointSession:
    """A checkpoint file plus the objects it stores (fields readable as attributes)."""

    def __init__(self, file, state):
        self.file = file
        self._state = dict(state)

    def __getattr__(self, name):
        st = self.__dict__.get("_state", {})
        if name in st:
            return st[name]
        raise AttributeError(name)


def _write(file, payload):
    tmp = file + ".tmp"
    with open(tmp, "wb") as f:
        pickle.dump(payload, f, protocol=pickle.HIGHEST_PROTOCOL)
        f.flush()
        os.fsync(f.fileno())
    os.replace(tmp, file)  # atomic, as tmp + mv
    return file


def init_checkpoint(file, **state):
    """Create a session storing `state` (device objects and plain values) and write it."""
    ckpt = CheckpointSession(file, state)
    checkpoint_(ckpt)
    return ckpt


def checkpoint_(ckpt, **overrides):
    """Export the stored objects (keywords override same-named entries) and write the
    file atomically."""
    ckpt._state.update(overrides)
    payload = {k: export_state(v) for k, v in ckpt._state.items()}
    return _write(ckpt.file, payload)


def restore_checkpoint(path, ctx=None):
    """Read a checkpoint and rebuild its objects on the device."""
    with open(path, "rb") as f:
        payload = pickle.load(f)
    return CheckpointSession(path, {k: import_state(v, ctx) for k, v in payload.items()})


def finalize_(ckpt):
    """Remove the checkpoint file (after a run completed)."""
    try:
        os.remove(ckpt.file)
    except FileNotFoundError:
        pass
