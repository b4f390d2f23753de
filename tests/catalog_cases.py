"""The catalog-ingestion fixtures (tests/golden/catalog_*.npz, made by TreeCorr's own Catalog
through tests/golden/make_catalog_golden.py): inputs, configuration and the reference's
results."""
import glob
import json
import os

import numpy as np

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
NAMES = sorted(os.path.basename(p)[8:-4] for p in glob.glob(os.path.join(HERE, "catalog_*.npz")))
VALUE_COLS = ("x", "y", "z", "ra", "dec", "r", "k", "g1", "g2")


def load(name):
    g = np.load(os.path.join(HERE, "catalog_%s.npz" % name))
    cfg = json.loads(str(g["config"]))
    inp = {k[3:]: g[k] for k in g.files if k.startswith("in_")}
    out = {k[4:]: g[k] for k in g.files if k.startswith("out_")}
    ref = dict(sumw=float(g["sumw"]), ntot=int(g["ntot"]), nobj=int(g["nobj"]),
               nontrivial_w=bool(g["nontrivial_w"]), center_size=g["center_size"])
    return cfg, inp, out, ref


def split_inputs(inp):
    """(value columns, w, wpos, flag) of a fixture's inputs."""
    cols = {k: v for k, v in inp.items() if k in VALUE_COLS}
    return cols, inp.get("w"), inp.get("wpos"), inp.get("flag")


def flag_args(cfg):
    return dict(ignore_flag=cfg.get("ignore_flag"), ok_flag=cfg.get("ok_flag", 0),
                keep_zero_weight=cfg.get("keep_zero_weight", False))
