"""Checkpoint / restart files of the GB300 path.

The reference writes its restart data through OPS's HDF5 layer: every time-advance array
(rho_B0, rhou0_B0, ..., rhoE_B0) as a dataset of the block group with the OPS attributes
(d_m / d_p halo depths, size, base, block_index, type; utilities/helperfunctions.py:99-147), and
the constants ``simulation_time`` and ``iter``; a restarted run reads them back with
``ops_decl_dat_hdf5`` / ``ops_get_const_hdf5`` (code_generation/opsc.py:962-977, 1198-1252).
Neither HDF5 nor h5py exists where this package runs, so the same content goes into one .npz:

* ``<block>/<name>_B<b>``: each conserved variable, the whole allocation in OPS layout (x
  fastest, the 5-point halos included), FP64;
* ``<block>/<name>_RKold_B<b>``: the RK register of that variable (the low-storage register,
  or the SBLI step-start copy), so a file written between any two steps restarts exactly;
* ``meta``: JSON with ``iter``, ``simulation_time`` and, per dataset, the OPS attributes
  (``d_m``, ``d_p``, ``size``, ``base``, ``block_index``, ``type``) and the block's spec record.

Restarting from such a file continues bit for bit like the run that wrote it.
"""
import json

import numpy as np

FORMAT = "opensbli_gb300 restart 1"


def dataset_names(ndim, b):
    """Conserved-variable dataset names of block b (the generated code's dat names)."""
    return ["rho_B%d" % b] + ["rhou%d_B%d" % (i, b) for i in range(ndim)] + ["rhoE_B%d" % b]


def write(path, specs, states, registers, iteration, simulation_time, block_names=None):
    """Write a restart file: specs (BlockSpec per block), states / registers ([nvars arrays] per
    block, OPS layout with halos), the iteration count and the simulation time."""
    arrays = {}
    meta = {"format": FORMAT, "iter": int(iteration), "simulation_time": float(simulation_time), "blocks": []}
    for b, spec in enumerate(specs):
        group = block_names[b] if block_names else "opensbliblock%02d" % b
        names = dataset_names(spec.ndim, b)
        if len(states[b]) != spec.nvars or len(registers[b]) != spec.nvars:
            raise ValueError("block %d: %d variables expected" % (b, spec.nvars))
        rec, _ = spec.to_record()
        entry = {"group": group, "spec": rec, "datasets": {}}
        for v, name in enumerate(names):
            for key, arr in ((name, states[b][v]), (name.replace("_B", "_RKold_B"), registers[b][v])):
                a = np.ascontiguousarray(arr, dtype=np.float64)
                if a.shape != tuple(spec.shape):
                    raise ValueError("%s: shape %s, the block allocation is %s" % (key, a.shape, spec.shape))
                arrays["%s/%s" % (group, key)] = a
                entry["datasets"][key] = {"d_m": [-spec.halo] * spec.ndim, "d_p": [spec.halo] * spec.ndim,
                                          "size": [int(n) for n in spec.size[:spec.ndim]],
                                          "base": [0] * spec.ndim, "block_index": b, "type": "double"}
        meta["blocks"].append(entry)
    np.savez(path, meta=np.array(json.dumps(meta)), **arrays)


def read(path):
    """Read a restart file: dict with "iter", "simulation_time", "blocks" (per block: "group",
    "spec" record, "state" and "register" lists of arrays)."""
    with np.load(path) as f:
        meta = json.loads(str(f["meta"]))
        if meta.get("format") != FORMAT:
            raise ValueError("%s is not a restart file of this package" % path)
        blocks = []
        for b, entry in enumerate(meta["blocks"]):
            nd = entry["spec"]["ndim"]
            names = dataset_names(nd, b)
            g = entry["group"]
            blocks.append({"group": g, "spec": entry["spec"],
                           "state": [f["%s/%s" % (g, n)] for n in names],
                           "register": [f["%s/%s" % (g, n.replace("_B", "_RKold_B"))] for n in names]})
    return {"iter": meta["iter"], "simulation_time": meta["simulation_time"], "blocks": blocks}


def check_compatible(specs, data):
    """Raise ValueError unless the file's blocks have the sizes and discretisation of specs."""
    if len(data["blocks"]) != len(specs):
        raise ValueError("restart file has %d blocks, the run %d" % (len(data["blocks"]), len(specs)))
    for b, (spec, blk) in enumerate(zip(specs, data["blocks"])):
        rec = blk["spec"]
        if tuple(rec["size"]) != tuple(spec.size) or rec["ndim"] != spec.ndim or rec["halo"] != spec.halo:
            raise ValueError("block %d: restart file size %s, the run's %s" % (b, rec["size"], spec.size))
        for k in ("scheme", "averaging", "viscous", "split_form", "filter", "flux_type"):
            if rec[k] != getattr(spec, k):
                raise ValueError("block %d: restart file %s %s, the run's %s" % (b, k, rec[k], getattr(spec, k)))
