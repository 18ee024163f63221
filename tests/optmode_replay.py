"""Replays of the kernel-dispatch calls recorded from the unmodified reference
(tests/golden/optmode.npz, written by make_golden.py's ``optmode`` group).

Each record holds a kernel name (the reference's optimization-module name,
``transforms.*`` for the recursive Legendre transforms), its arguments before
the call and the arrays the call wrote.  ``calls()`` rebuilds the arguments
(numpy copies, or CUDA tensors with ``device=True``) so that a test can feed
them to another implementation and compare what it writes.
"""
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PATH = os.path.join(HERE, "golden", "optmode.npz")


class Record:
    def __init__(self, name, args, outputs):
        self.name = name
        self.args = args          # rebuilt arguments
        self.outputs = outputs    # {arg index: recorded array after the call}

    def rel_errors(self):
        """Relative max-norm error of every written argument against the record."""
        errs = {}
        for j, ref in self.outputs.items():
            got = self.args[j]
            if hasattr(got, "detach"):
                got = got.detach().cpu().numpy()
            got = np.asarray(got)
            scale = max(np.abs(ref).max(), 1e-300)
            errs[j] = float(np.abs(got - ref).max() / scale)
        return errs


def calls(device=False, names=None):
    z = np.load(PATH)
    manifest = json.loads(str(z["manifest"]))
    out = []
    for c in manifest:
        if names is not None and c["name"] not in names:
            continue
        args, outputs = [], {}
        for j, s in enumerate(c["args"]):
            t = s["t"]
            if t == "arr":
                a = np.array(z[s["key"]], copy=True)
                if device:
                    import torch
                    a = torch.from_numpy(a).to("cuda")
                args.append(a)
                if "out" in s:
                    outputs[j] = np.array(z[s["out"]])
            elif t == "mat":
                args.append({o: np.array(z[f"{s['key']}_d{o}"]) for o in s["offsets"]})
            elif t == "num":
                args.append(int(s["v"]) if s.get("int") else s["v"])
            elif t == "bool":
                args.append(s["v"])
            elif t == "fn":
                args.append(s["v"])  # a function name: the caller resolves it
            else:
                raise ValueError(t)
        out.append(Record(c["name"], args, outputs))
    return out
