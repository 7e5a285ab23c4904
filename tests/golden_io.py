"""Loading helpers for the golden fixtures made by tests/golden/make_golden.py."""
import ast
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _pair_tables(z):
    tabs = []
    for k in range(int(z["npair"])):
        g = z[f"pair{k}_grid"]
        p = z[f"pair{k}_params"]
        tabs.append(dict(species=tuple(int(v) for v in z[f"pair{k}_species"]),
                         ngpts=int(g[0]), norder=int(g[1]), rgridinv=float(p[0]),
                         logrratioinv=float(p[1]), ugrid=z[f"pair{k}_ugrid"]))
    return tabs


def load_tables(name):
    """Pair tables pi-qmc built for a configuration (tables_<name>.npz)."""
    z = np.load(os.path.join(GOLDEN, "tables_" + name + ".npz"))
    return dict(kw=ast.literal_eval(str(z["config"])), tables=_pair_tables(z))


def load(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    kw = ast.literal_eval(str(z["config"]))
    tabs = _pair_tables(z)
    ew = None
    if "ewald_kvec" in z:
        ew = dict(totk=len(z["ewald_vk"]), kvec=z["ewald_kvec"], vk=z["ewald_vk"],
                  one_over_2v=float(z["ewald_scalars"][0]),
                  self_energy=float(z["ewald_scalars"][1]),
                  ikmax=[int(v) for v in z["ewald_ikmax"]], coef=z["ewald_coef"])
    rec = {k: z["rec_" + k] for k in ("ifirst1", "ifirst2", "ipart", "reject_level", "ds",
                                      "ds_node", "lnt")}
    est = {}
    if "est_virial" in z:
        est["virial"] = dict(zip((int(w) for w in z["est_virial_windows"]),
                                 (float(v) for v in z["est_virial"])))
        est["coulomb"] = float(z["est_coulomb"])
    if "estew_kvec" in z:
        prm = z["estew_params"]
        est["ewald"] = dict(epsilon=float(prm[0]), rcut=float(prm[1]), kcut=float(prm[2]),
                            table=dict(totk=len(z["estew_vk"]), kvec=z["estew_kvec"],
                                       vk=z["estew_vk"],
                                       one_over_2v=float(z["estew_scalars"][0]),
                                       self_energy=float(z["estew_scalars"][1]),
                                       ikmax=[int(v) for v in z["estew_ikmax"]]),
                            vgrid=z["estew_vgrid"], energy=float(z["est_ewald_coulomb"]))
    disp = None
    if "disp_params" in z:
        prm = z["disp_params"]
        disp = dict(box=[float(v) for v in prm[:3]], nmoving=int(prm[3]), species=int(prm[4]),
                    nattempt=int(prm[5]), first_attempt=int(prm[6]),
                    records={k: z["disp_" + k] for k in ("ipart", "disp", "ds", "ds_node",
                                                         "accepted")},
                    path=z["path0"] + z["dpath"] + z["disp_dpath"])
    return dict(kw=kw, tables=tabs, ewald=ew, path0=z["path0"], estimators=est, displace=disp,
                path1=z["path0"] + z["dpath"], energy0=float(z["energy0"]),
                energy1=float(z["energy1"]), records=rec, nattempt=int(z["nattempt"]),
                naccepted=int(z["naccepted"]))


def load_nodes(name):
    """NodeModel fixture of a case: slice pairs r1, r2 [nb][npart][3] and, per
    node species sp, pi-qmc's scale, err, det, d1, d2 (and for the SHO dot at
    omega/T = 20 the 60-digit values exact_det, exact_d1, exact_d2 over the
    species' own particles, which start at index `first`)."""
    z = np.load(os.path.join(GOLDEN, "nodes_" + name + ".npz"))
    kw = ast.literal_eval(str(z["config"]))
    out = dict(kw=kw, r1=z["r1"], r2=z["r2"], species={})
    for sp in range(len(kw["counts"])):
        if f"sp{sp}_det" not in z:
            continue
        d = {k: z[f"sp{sp}_{k}"] for k in ("err", "det", "d1", "d2")}
        d["scale"] = float(z[f"sp{sp}_scale"])
        if f"sp{sp}_exact_det" in z:
            d.update(exact_det=z[f"sp{sp}_exact_det"], exact_d1=z[f"sp{sp}_exact_d1"],
                     exact_d2=z[f"sp{sp}_exact_d2"], first=int(z[f"sp{sp}_first"]))
        out["species"][sp] = d
    return out
