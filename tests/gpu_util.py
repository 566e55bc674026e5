"""Run one specialization on the GPU through the kernel table (torch tensors)."""

import numpy as np

from awkward_gb300._signatures import SIGNATURES

NP = {
    "bool": np.bool_, "int8_t": np.int8, "uint8_t": np.uint8, "int16_t": np.int16,
    "uint16_t": np.uint16, "int32_t": np.int32, "uint32_t": np.uint32,
    "int64_t": np.int64, "uint64_t": np.uint64, "float": np.float32, "double": np.float64,
}


def to_dev(a, base):
    import torch

    a = np.ascontiguousarray(np.asarray(a, dtype=NP[base]))
    return torch.from_numpy(a.copy()).to("cuda")


def run_gpu(name, kw):
    """Returns (outputs as numpy, error string or None)."""
    import awkward_gb300

    be = awkward_gb300.backend()
    kern = be.by_name(name)
    targs, dev = [], {}
    for (an, base, _d, depth, _c, _r) in SIGNATURES[name]["args"]:
        v = kw[an]
        if depth == 0:
            targs.append(v)
        elif depth == 1:
            dev[an] = to_dev(v, base)
            targs.append(dev[an])
        else:
            dev[an] = [to_dev(r, base) for r in v]
            targs.append(dev[an])
    err = None
    kern(*targs)
    try:
        be.synchronize()
    except ValueError as e:
        err = str(e)
    outs = {}
    for an, t in dev.items():
        outs[an] = [r.cpu().numpy() for r in t] if isinstance(t, list) else t.cpu().numpy()
    return outs, err
