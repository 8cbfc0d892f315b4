"""ctypes mirror of the parsed deck (include/mpm_deck.h: mpm_deck,
mpm_material, mpm_body) for tests that compare two parses field by field.
Only tests use it; the library's bindings go through plain accessors."""
import ctypes

import numpy as np


class Material(ctypes.Structure):
    _fields_ = [("mat_type", ctypes.c_int32), ("eos_type", ctypes.c_int32)] + [
        (n, ctypes.c_double) for n in ("density", "miu", "young", "poisson", "yield0", "tangmod", "roomt",
                                       "melt", "specheat", "B_jc", "n_jc", "C_jc", "m_jc", "epso", "prd", "epf",
                                       "D")] + [
        ("cEos", ctypes.c_double * 10)] + [
        (n, ctypes.c_double) for n in ("wavespd", "bulk_modulus", "q_fai", "k_fai", "q_psi", "ten_f")]


class Body(ctypes.Structure):
    _fields_ = [("mat", ctypes.c_int32), ("comID", ctypes.c_int32), ("gravp", ctypes.c_double * 3),
                ("par_begin", ctypes.c_int64), ("par_end", ctypes.c_int64)]


MAX_DETO, MAX_CURVES, MAX_ANIM = 10, 64, 64


class DeckStruct(ctypes.Structure):
    _fields_ = [
        ("title", ctypes.c_char * 257), ("nb_particle", ctypes.c_int64),
        ("nb_component", ctypes.c_int32), ("nb_body", ctypes.c_int32), ("nb_mat", ctypes.c_int32),
        ("flags", ctypes.c_int32), ("mats", ctypes.POINTER(Material)), ("bodies", ctypes.POINTER(Body)),
        ("mass", ctypes.POINTER(ctypes.c_double)), ("xp", ctypes.POINTER(ctypes.c_double)),
        ("vxp", ctypes.POINTER(ctypes.c_double)), ("fxp", ctypes.POINTER(ctypes.c_double)),
        ("skip", ctypes.POINTER(ctypes.c_uint8)), ("span", (ctypes.c_double * 2) * 3),
    ] + [(n, ctypes.c_double) for n in ("dcell", "cutoff", "dtscale", "endtime", "outtime", "reporttime",
                                        "quasi_load_time", "damp_factor", "bq1", "bq2")] + [
        ("fixs", ctypes.c_int32 * 6), ("contact_type", ctypes.c_int32), ("normbody", ctypes.c_int32),
        ("fricfa", ctypes.c_double), ("n_deto", ctypes.c_int32), ("deto", (ctypes.c_double * 3) * MAX_DETO),
        ("n_curves", ctypes.c_int32), ("n_anim", ctypes.c_int32),
        ("curve_option", ctypes.c_int32 * MAX_CURVES), ("curve_point", ctypes.c_int32 * MAX_CURVES),
        ("anim_option", ctypes.c_int32 * MAX_ANIM), ("plot2d", ctypes.c_double * 6),
        ("line_nb", ctypes.c_int32), ("err", ctypes.c_char * 256),
    ]


def deck_record(deck) -> dict:
    """Every parsed value of a deck (mpm3d_gb300.Deck) as plain Python /
    numpy values, except the title and the reader's bookkeeping (last line
    number, error text)."""
    d = ctypes.cast(deck.handle, ctypes.POINTER(DeckStruct)).contents
    n = d.nb_particle
    out = {}
    for name, _ in DeckStruct._fields_:
        if name in ("title", "line_nb", "err", "mats", "bodies", "mass", "xp", "vxp", "fxp", "skip"):
            continue
        v = getattr(d, name)
        if isinstance(v, ctypes.Array):
            v = np.ctypeslib.as_array(v).copy()
        out[name] = v
    for name, comp in (("mass", 1), ("xp", 3), ("vxp", 3), ("fxp", 3)):
        out[name] = np.ctypeslib.as_array(getattr(d, name), shape=(comp * n,)).copy()
    out["skip"] = np.ctypeslib.as_array(d.skip, shape=(n,)).copy() if d.skip else None
    out["mats"] = [{f: (np.ctypeslib.as_array(getattr(d.mats[k], f)).copy()
                        if f == "cEos" else getattr(d.mats[k], f)) for f, _ in Material._fields_}
                   for k in range(d.nb_mat)]
    out["bodies"] = [{f: (list(getattr(d.bodies[k], f)) if f == "gravp" else getattr(d.bodies[k], f))
                      for f, _ in Body._fields_} for k in range(d.nb_body)]
    return out


def diff_records(a: dict, b: dict) -> list:
    """Names of the entries that differ (bit for bit for reals)."""
    bad = []
    for k in a:
        x, y = a[k], b[k]
        if k in ("mats", "bodies"):
            if len(x) != len(y):
                bad.append(k)
                continue
            for i, (p, q) in enumerate(zip(x, y)):
                for f in p:
                    if not np.array_equal(np.asarray(p[f]), np.asarray(q[f])):
                        bad.append(f"{k}[{i}].{f}")
        elif x is None or y is None:
            if (x is None) != (y is None):
                bad.append(k)
        elif not np.array_equal(np.asarray(x), np.asarray(y)):
            bad.append(k)
    return bad
