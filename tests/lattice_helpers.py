"""Builds the lattice golden models with the engine's lattice layer."""
from models import LATTICE_CASES, hubbard_cluster


def build_lattice(tag):
    import pyqcm_gb300 as pg
    from pyqcm_gb300.lattice import LatticeModel
    c = LATTICE_CASES[tag]
    ns, nb = len(c["sites"]), c["n_bath"]
    cm = pg.ClusterModel(ns, nb)
    if nb:
        _, _, bops = hubbard_cluster(2, 2, nb)
        for op, (typ, els) in bops.items():
            if op.startswith("eb") or op.startswith("tb"):
                cm.new_operator(op, typ, els)
    lm = LatticeModel(cm, c["sites"], c["superlattice"])
    for op in c["ops"]:
        if op[0] == "inter":
            lm.interaction_operator(op[1], op[2])
        elif op[0] == "hop":
            lm.hopping_operator(op[1], op[2], op[3], tau=op[4], sigma=op[5])
        elif op[0] == "dw":
            lm.density_wave(op[1], op[2], op[3], op[4], op[5])
    lm.set_target_sectors(c["sector"])
    lm.set_parameters(c["params"])
    return lm
