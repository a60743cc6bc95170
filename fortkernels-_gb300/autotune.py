"""Work-shape tuner for the batched GPP forms.

Tiles.  
Each work item of the main pass covers a (band block x column block x
g-vector split) tile.  Two kernel families are compiled: the shared-frequency kernel (every band uses the same three
frequencies, the mini-app's case): 64 bands x 32 columns, 32 x 64, 32 x 32,
64 x 16 (tiles 3, 4, 5, 6; a batch whose instances all take 5 or 6 runs two
CTAs per SM); and the per-band-frequency kernel: 32 x 32,
16 x 64, 64 x 16 (tiles 0, 1, 2).  Which shape is fastest depends on how the
instance's number_bands and ngpown pad to the block sizes and on how much
staged data each item re-reads, so the choice is made per shape class:

    class "b{i}c{j}":  i = ((ceil(number_bands / 16) - 1) mod 4),
                       j = ((ceil(ngpown / 16) - 1) mod 4)

i.e. how many 16-band (16-column) slabs the last 64-wide block holds.  The
tuner times every tile of both families on one representative instance per
class (nc = 4096; all tiles scale the same way in ncouls) through a
one-instance batch replayed as a CUDA graph, and writes the fastest tile per
class and family to `tuning/gpp_tiles_gb300.json`.  `tile_for()` reads that
table; without it the library picks the least-padded tile itself.

Sizing.  The g-vector split of every form's work items is set by how many
items each resident CTA takes (sigma_gpp_batch_create_tuned): the FP64 and
mixed main passes' items per CTA (band block x column block x g-vector
split), and the tensor form's contraction item length (the K split of every
instance's 128-row x 64-band blocks; 0 sizes each instance as its single
plan).  The tuner times each candidate
on the 48-instance set through graph replays and keeps the fastest; a
tensor candidate is kept only if every achtemp / asxtemp of the set stays
within 1e-6 of the FP64 form's (the tensor form's error depends on where
its K splits fall, so a subset does not decide it).
`sizing_for(form)` reads the choice (0 = the library's default).

    python fortkernels-_gb300/autotune.py --out <path>
"""
from __future__ import annotations

import argparse
import json
import pathlib

PKG = pathlib.Path(__file__).resolve().parent
TABLE = PKG / "tuning" / "gpp_tiles_gb300.json"
TILES = {0: "32x32", 1: "16x64", 2: "64x16", 3: "y64x32", 4: "y32x64", 5: "y32x32", 6: "y64x16"}
FAMILIES = {"shared": (3, 4, 5, 6), "per_band": (0, 1, 2)}
TABLE_KEY = {"shared": "classes", "per_band": "classes_per_band"}
_table = None


def shape_class(number_bands: int, ngpown: int) -> str:
    i = ((number_bands + 15) // 16 - 1) % 4
    j = ((ngpown + 15) // 16 - 1) % 4
    return f"b{i}c{j}"


def load_table(path=None):
    global _table
    if path is None and _table is not None:
        return _table
    p = pathlib.Path(path) if path else TABLE
    t = json.loads(p.read_text()) if p.exists() else None
    if path is None:
        _table = t
    return t


def tile_for(number_bands: int, ngpown: int, table=None, shared=True) -> int:
    """Tuned tile for this shape and kernel family (-1 = the library's
    least-padding choice)."""
    t = table if table is not None else load_table()
    if not t or TABLE_KEY["shared" if shared else "per_band"] not in t:
        return -1
    v = int(t[TABLE_KEY["shared" if shared else "per_band"]].get(shape_class(number_bands, ngpown), -1))
    return v if v in FAMILIES["shared" if shared else "per_band"] else -1


SIZING_INSTANCES = 48
SIZING_CANDIDATES = {"fp64": (8, 16, 32), "mixed": (8, 16, 32), "tensor": (0, 32, 64, 128)}
SIZING_KEY = {"fp64": "fp64_items_per_cta", "mixed": "mixed_items_per_cta", "tensor": "tensor_split_tiles"}


def sizing_for(form: str, table=None) -> int:
    """Tuned sizing of a batched form: items per CTA ("fp64", "mixed") or
    the contraction items' K tiles ("tensor"); 0 selects the library's
    default."""
    t = table if table is not None else load_table()
    if not t:
        return 0
    return int(t.get(SIZING_KEY[form], 0))


def _time_batch(S, torch, dicts, prec, stream, reps, tiles=None, ipc=0, tsplit=0):
    b = S.GppBatch(dicts, precision=prec, tiles=tiles, items_per_cta=ipc, tensor_split_tiles=tsplit)
    b.launch_graph(stream.cuda_stream)  # capture + warm-up
    b.launch_graph(stream.cuda_stream)
    stream.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        b.launch_graph(stream.cuda_stream)
    e1.record(stream)
    stream.synchronize()
    st = b.status(stream.cuda_stream)
    b.close()
    if st != 0:
        raise RuntimeError(f"batch status {st} in tuning")
    return e0.elapsed_time(e1) / reps


def tune_sizing(classes, reps=3, log=print):
    """Items per CTA of each batched form on the first SIZING_INSTANCES
    instances of the 48-instance set (all of them; FP64 with its tuned
    tiles)."""
    import numpy as np
    import torch

    import batched
    import sigma_gb300 as S
    import workload as W

    xs = batched.device_instances(W.batched_shapes()[:SIZING_INSTANCES])
    dicts = [x.as_dict() for x in xs]
    tiles = [tile_for(x.nb, x.ng, {"classes": classes}, shared=True) for x in xs]
    stream = torch.cuda.Stream()
    out, timings = {}, {}
    ref = None
    for form, prec in (("fp64", S.PREC_FP64), ("mixed", S.PREC_MIXED), ("tensor", S.PREC_TENSOR)):
        ms = {}
        for c in SIZING_CANDIDATES[form]:
            kw = dict(tsplit=c) if form == "tensor" else dict(ipc=c)
            ms[c] = _time_batch(S, torch, dicts, prec, stream, 1 if form == "fp64" else reps,
                                tiles=tiles if form == "fp64" else None, **kw)
            outs = [x.outputs() for x in xs]
            if form == "fp64" and ref is None:
                ref = outs
            if form == "tensor":
                worst = max(float(np.max(np.abs(o[k] - r[k]) / np.abs(r[k])))
                            for o, r in zip(outs, ref) for k in (0, 1))
                if worst > 1e-6:
                    log("tensor", c, "rejected: worst output", worst)
                    ms[c] = float("inf")
        best = min(ms, key=ms.get)
        out[SIZING_KEY[form]] = best
        timings[form] = {str(k): (round(v, 4) if v != float("inf") else None) for k, v in ms.items()}
        log("sizing", form, timings[form], "->", best)
    del xs, dicts
    torch.cuda.empty_cache()
    out["sizing_timings_ms"] = timings
    out["sizing_instances"] = SIZING_INSTANCES
    return out


def representative(cls_i: int, cls_j: int):
    """number_bands, ngpown of the class's representative instance."""
    return 256 + 16 * cls_i + 9, 512 + 16 * cls_j + 9


def tune(reps=5, ncouls=4096, log=print):
    import torch

    import batched
    import sigma_gb300 as S

    S.load()
    stream = torch.cuda.Stream()
    out = {"version": 3, "device": torch.cuda.get_device_name(),
           "tiles": {str(k): v for k, v in TILES.items()},
           "class_rule": "b{i}c{j}: i = (ceil(number_bands/16)-1) mod 4, j = (ceil(ngpown/16)-1) mod 4"}
    for family, tiles in FAMILIES.items():
        classes, timings = {}, {}
        for i in range(4):
            for j in range(4):
                nb, ng = representative(i, j)
                key = shape_class(nb, ng)
                inst = batched.DeviceInstance(nb, 2, ncouls, ng, seed=5000 + 4 * i + j,
                                              per_band_wx=family == "per_band")
                ms = {}
                for tile in tiles:
                    ms[TILES[tile]] = _time_batch(S, torch, [inst.as_dict()], S.PREC_FP64, stream, reps,
                                                  tiles=[tile])
                best = min(ms, key=ms.get)
                classes[key] = [k for k, v in TILES.items() if v == best][0]
                timings[key] = {"number_bands": nb, "ngpown": ng, "ncouls": ncouls,
                                "ms": {k: round(v, 4) for k, v in ms.items()}}
                log(family, key, nb, ng, {k: round(v, 3) for k, v in ms.items()}, "->", best)
                del inst
                torch.cuda.empty_cache()
        out[TABLE_KEY[family]] = classes
        out["timings" if family == "shared" else "timings_per_band"] = timings
    out.update(tune_sizing(out["classes"], log=log))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=str(TABLE))
    ap.add_argument("--reps", type=int, default=5)
    a = ap.parse_args()
    t = tune(a.reps)
    out = pathlib.Path(a.out)
    out.parent.mkdir(parents=True, exist_ok=True)
    out.write_text(json.dumps(t, indent=1) + "\n")
    print(f"wrote {out}")


if __name__ == "__main__":
    import sys
    for p in (str(PKG), str(PKG.parent)):
        if p not in sys.path:
            sys.path.insert(0, p)
    main()
