"""ctypes mirror of the C ABI structs of ``include/esmcuda.h`` and their construction from a
:class:`~esmgb.model.SynthModel`.

The same ``esm_model`` struct is what a Julia ``ccall`` shim would fill from the reference's
``EnergyModel``/``LocalModel``; here it is filled from the synthetic model.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from .model import FAMILY_RATES, SynthModel

P_i32 = C.POINTER(C.c_int32)
P_f64 = C.POINTER(C.c_double)
NFAM = 11


class EsmModel(C.Structure):
    _fields_ = [
        ("N", C.c_int32), ("L", C.c_int32), ("T", C.c_int32), ("dt", C.c_double),
        ("bus0", P_i32), ("bus1", P_i32), ("line_b", P_f64), ("line_s", P_f64),
        ("K", C.c_int32),
        ("unit_kind", P_i32), ("unit_group", P_i32), ("unit_bus", P_i32), ("unit_series", P_i32),
        ("unit_mc", P_f64), ("unit_capex", P_f64), ("unit_lo", P_f64), ("unit_hi", P_f64), ("unit_avail", P_f64),
        ("unit_hours", P_f64), ("unit_eta_in", P_f64), ("unit_eta_out", P_f64), ("unit_qt", P_f64),
        ("D", C.c_int32), ("S", C.c_int32), ("disp", P_i32), ("stor", P_i32),
        ("n0", C.c_int32), ("nreg", C.c_int32), ("series_field", P_i32), ("series_node", P_i32),
        ("xbar", P_f64), ("wscale", P_f64), ("Ptr", P_f64), ("pi0", P_f64), ("phi", P_f64), ("mu", P_f64),
        ("sig", P_f64), ("sig0", P_f64),
        ("c_shed", C.c_double), ("c_dump", C.c_double), ("c_viol", C.c_double), ("gamma_k", C.c_double),
        ("kappa0", C.c_double), ("beta_v", C.c_double), ("beta_k", C.c_double), ("physical", C.c_int32),
        ("nfields", C.c_int32), ("field_role", P_i32), ("field_atom_ptr", P_i32), ("atom_ptr", P_i32),
        ("atom_idx", P_i32), ("atom_val", P_f64),
        ("nodelines_ptr", P_i32), ("nodelines", P_i32), ("units_ptr", P_i32), ("units_at", P_i32),
        ("stor_ptr", P_i32), ("stor_at", P_i32),
        ("nlev", C.c_int32), ("qcum", P_f64), ("cell_level_ptr", P_i32), ("cell_ptr", P_i32), ("cell_units", P_i32),
        ("xpart_ptr", P_i32), ("xpart", P_i32), ("xnod_ptr", P_i32), ("xnod", P_i32), ("xval", P_f64),
        ("xlk_ptr", P_i32), ("xlkn", P_i32), ("xlkg", P_f64),
        ("reroute", P_f64), ("comp", P_i32),
        ("nsgroups", C.c_int32), ("sgroup_ptr", P_i32), ("sgroup_units", P_i32),
    ]


class EsmOpts(C.Structure):
    _fields_ = [
        ("R", C.c_int32), ("precision", C.c_int32), ("seed", C.c_uint64), ("extra", C.c_double),
        ("maxnats", C.c_double), ("kappa_min", C.c_double), ("max_points", C.c_int32), ("span", C.c_int32),
        ("family_rates", C.c_double * NFAM), ("storage_ms", C.c_int32), ("storage_long", C.c_int32),
        ("probe", C.c_int32),
    ]


def _i32(a):
    return np.ascontiguousarray(np.asarray(a), dtype=np.int32)


def _f64(a):
    return np.ascontiguousarray(np.asarray(a), dtype=np.float64)


class ModelBuffers:
    """Owns the numpy arrays behind an :class:`EsmModel` (keep it alive while the struct is used)."""

    def __init__(self, m: SynthModel):
        keep = []

        def ip(a):
            a = _i32(a)
            keep.append(a)
            return a.ctypes.data_as(P_i32)

        def fp(a):
            a = _f64(a)
            keep.append(a)
            return a.ctypes.data_as(P_f64)

        fap = np.cumsum([0] + [len(a.ptr) - 1 for a in m.atoms])
        aptr, aidx, aval = [0], [], []
        for a in m.atoms:
            base = aptr[-1]
            aptr.extend((base + a.ptr[1:]).tolist())
            aidx.extend(a.idx.tolist())
            aval.extend(a.val.tolist())
        s = EsmModel()
        s.N, s.L, s.T, s.dt = m.N, m.L, m.T, m.dt
        s.bus0, s.bus1, s.line_b, s.line_s = ip(m.bus0), ip(m.bus1), fp(m.line_b), fp(m.line_s)
        s.K = m.Kunits
        s.unit_kind, s.unit_group, s.unit_bus, s.unit_series = ip(m.unit_kind), ip(m.unit_group), ip(m.unit_bus), ip(m.unit_series)
        s.unit_mc, s.unit_capex, s.unit_lo, s.unit_hi = fp(m.unit_mc), fp(m.unit_capex), fp(m.unit_lo), fp(m.unit_hi)
        s.unit_avail, s.unit_hours, s.unit_eta_in = fp(m.unit_avail), fp(m.unit_hours), fp(m.unit_eta_in)
        s.unit_eta_out, s.unit_qt = fp(m.unit_eta_out), fp(m.unit_qt)
        s.D, s.S, s.disp, s.stor = m.D, m.S, ip(m.disp), ip(m.stor)
        s.n0, s.nreg = m.n0, m.K
        s.series_field, s.series_node = ip(m.series_field), ip(m.series_node)
        s.xbar, s.wscale, s.Ptr, s.pi0 = fp(m.xbar.ravel()), fp(m.wscale), fp(m.Ptr.ravel()), fp(m.pi0)
        s.phi, s.mu, s.sig, s.sig0 = fp(m.phi.ravel()), fp(m.mu.ravel()), fp(m.sig.ravel()), fp(m.sig0)
        s.c_shed, s.c_dump, s.c_viol, s.gamma_k = m.c_shed, m.c_dump, m.c_viol, m.gamma_k
        s.kappa0, s.beta_v, s.beta_k, s.physical = m.kappa0, m.beta_v, m.beta_k, int(m.physical)
        s.nfields = len(m.atoms)
        s.field_role = ip([a.role for a in m.atoms])
        s.field_atom_ptr, s.atom_ptr, s.atom_idx, s.atom_val = ip(fap), ip(aptr), ip(aidx), fp(aval)
        s.nodelines_ptr, s.nodelines = ip(m.nodelines_ptr), ip(m.nodelines)
        s.units_ptr, s.units_at, s.stor_ptr, s.stor_at = ip(m.units_ptr), ip(m.units_at), ip(m.stor_ptr), ip(m.stor_at)
        s.nlev, s.qcum = len(m.qcum), fp(m.qcum)
        s.cell_level_ptr, s.cell_ptr, s.cell_units = ip(m.cell_level_ptr), ip(m.cell_ptr), ip(m.cell_units)
        s.xpart_ptr, s.xpart, s.xnod_ptr, s.xnod = ip(m.xpart_ptr), ip(m.xpart), ip(m.xnod_ptr), ip(m.xnod)
        s.xval, s.xlk_ptr, s.xlkn, s.xlkg = fp(m.xval), ip(m.xlk_ptr), ip(m.xlkn), fp(m.xlkg)
        s.reroute, s.comp = fp(m.reroute.ravel()), ip(m.comp)
        gptr, gunits = storage_groups(m)
        s.nsgroups, s.sgroup_ptr, s.sgroup_units = len(gptr) - 1, ip(gptr), ip(gunits)
        self.struct = s
        self._keep = keep
        self.natoms = int(fap[-1])


def probe_seed(seed):
    """esm_probe_seed: the seed of the lag probe's streams."""
    return int(seed) ^ 0x50524F4245000000


def storage_groups(m: SynthModel):
    """The cell-class aggregates of the storage multiscale sweep (src/flowmoves.jl:270-274): the
    storage units grouped by (country cell of their node, carrier), keys in sorted order, units in
    storage order; CSR (ptr, units as indices into stor)."""
    groups = {}
    for j, u in enumerate(m.stor):
        groups.setdefault((int(m.country[m.unit_bus[u]]), int(m.unit_group[u])), []).append(j)
    keys = sorted(groups)
    ptr = np.cumsum([0] + [len(groups[k]) for k in keys]).astype(np.int32)
    units = np.array([j for k in keys for j in groups[k]], np.int32)
    return ptr, units


def make_opts(R, precision=32, seed=1, extra=4.0, maxnats=40.0, kappa_min=1.0, max_points=0, span=0,
              rates=FAMILY_RATES, storage_ms=0, storage_long=0, probe=0) -> EsmOpts:
    o = EsmOpts()
    o.R, o.precision, o.seed, o.extra, o.maxnats, o.kappa_min = R, precision, seed, extra, maxnats, kappa_min
    o.max_points, o.span, o.storage_ms, o.storage_long = max_points, span, int(storage_ms), int(storage_long)
    o.probe = int(probe)
    for i, r in enumerate(rates):
        o.family_rates[i] = r
    return o
