"""Black-oil Newton Jacobian assembly on the device (``rsg_bo_*`` in include/rsg.h).

Mirror of the engine's assembly step, ``Simulator::evalAll`` + ``Simulator::assemble`` (engine/src/simulator.cpp:
2429-2459, 2500-3033): the reservoir terms of the fully implicit black-oil system at a state, written on the device
into the engine's scalar Jacobian layout, with the engine's well terms passed in as addends. The model description is
a dict with the engine's arrays (the keys of tests/golden/waterflood_asm.npz):

- grid: ``na``, ``nv``, ``nw``, ``adjStart``, ``adjNbr``, ``adjConn``, ``conn_a``, ``conn_trans``, ``conn_dDepth``,
  ``poreVolRef``, ``gravity``, ``vars`` (i_sw, i_x, eq[3]);
- pattern: ``J_rowPtr``, ``J_col`` (Simulator::buildPattern);
- fluid (ressim::FluidModel): ``phases`` (W, O, G, live, vap), ``pvtw``, ``rock``, ``rhoSC``, ``gasFactor``, the tables
  ``rsOfP``, ``pbOfRs``, ``deadB``, ``deadBMu``, ``gasB``, ``gasBMu`` (``<name>_x``, ``_y``, ``_clamp``), the live oil
  nodes ``liveRs``, ``bSat``, ``bmuSat`` and the undersaturated tables ``uB`` / ``uBMu`` (concatenated, ``_off``);
- saturation functions (ressim::SatFunctions): ``krw``, ``krow``, ``pcow``, ``krg``, ``krog``, ``pcog``, ``swco``,
  ``kroModel``, ``sat_flags`` (water, gas, three-point).

No CPU fallback: every call runs on the GPU through librsg.so.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def model_structs(model: dict):
    """The C-ABI descriptions of a model dict (rsg_bo_grid, rsg_bo_fluid, rsg_bo_satfun), the Jacobian pattern
    (int32 rowPtr, col) and the arrays they point into (keep them alive while the structures are used)."""
    keep = []

    def arr(a, conv):
        a = conv(a)
        keep.append(a)
        return C.c_void_p(a.ctypes.data) if a.size else None

    def table(name):
        x, y = _f64(model[name + "_x"]), _f64(model[name + "_y"])
        keep.extend([x, y])
        return _lib.Table(int(x.size), C.c_void_p(x.ctypes.data) if x.size else None,
                          C.c_void_p(y.ctypes.data) if y.size else None, int(np.asarray(model[name + "_clamp"]).ravel()[0]))

    def tables(name):
        x, y, off, cl = _f64(model[name + "_x"]), _f64(model[name + "_y"]), _i32(model[name + "_off"]), _i32(model[name + "_clamp"])
        keep.extend([x, y])
        ts = (_lib.Table * (off.size - 1))()
        for k in range(off.size - 1):
            ts[k] = _lib.Table(int(off[k + 1] - off[k]), C.c_void_p(x.ctypes.data + 8 * int(off[k])),
                               C.c_void_p(y.ctypes.data + 8 * int(off[k])), int(cl[k]))
        keep.append(ts)
        return C.cast(ts, C.c_void_p)

    sc = lambda k: np.asarray(model[k]).ravel()  # noqa: E731
    na, nv = int(sc("na")[0]), int(sc("nv")[0])
    v = sc("vars")
    g = _lib.BoGrid(na, nv, int(np.asarray(model["conn_trans"]).size), arr(model["adjStart"], _i32), arr(model["adjNbr"], _i32),
                    arr(model["adjConn"], _i32), arr(model["conn_a"], _i32), arr(model["conn_trans"], _f64),
                    arr(model["conn_dDepth"], _f64), arr(model["poreVolRef"], _f64), float(sc("gravity")[0]), int(v[0]), int(v[1]),
                    (C.c_int * 3)(int(v[2]), int(v[3]), int(v[4])))
    ph = sc("phases")
    f = _lib.BoFluid()
    f.water, f.oil, f.gas, f.live, f.vap = (int(t) for t in ph[:5])
    f.pvtw = (C.c_double * 5)(*sc("pvtw"))
    f.rock = (C.c_double * 2)(*sc("rock"))
    f.rho_sc = (C.c_double * 3)(*sc("rhoSC"))
    f.gas_factor = float(sc("gasFactor")[0])
    f.rs_of_p, f.pb_of_rs = table("rsOfP"), table("pbOfRs")
    f.dead_b, f.dead_bmu = table("deadB"), table("deadBMu")
    f.gas_b, f.gas_bmu = table("gasB"), table("gasBMu")
    f.nsat = int(np.asarray(model["liveRs"]).size)
    f.sat_rs, f.sat_b, f.sat_bmu = arr(model["liveRs"], _f64), arr(model["bSat"], _f64), arr(model["bmuSat"], _f64)
    f.under_b, f.under_bmu = tables("uB"), tables("uBMu")
    s = _lib.BoSatfun()
    s.krw, s.krow, s.pcow = table("krw"), table("krow"), table("pcow")
    s.krg, s.krog, s.pcog = table("krg"), table("krog"), table("pcog")
    s.swco = float(sc("swco")[0])
    s.kro_model = int(sc("kroModel")[0])
    sf = sc("sat_flags")
    s.water, s.gas, s.three_point = int(sf[0]), int(sf[1]), int(sf[2])
    rowPtr, col = _i32(model["J_rowPtr"]), _i32(model["J_col"])
    keep.extend([rowPtr, col])
    return g, f, s, rowPtr, col, keep


class BlackOilAssembler:
    """One grid's assembler on ``device``: ``assemble_device`` writes J and R into caller-owned device buffers."""

    def __init__(self, model: dict, device: int = 0):
        self._L = _lib.load()
        self._h = C.c_void_p()
        g, f, s, rowPtr, col, keep = model_structs(model)
        self.na, self.nv, self.nw = int(g.na), int(g.nv), int(np.asarray(model["nw"]).ravel()[0])
        self.nrows = self.na * self.nv + self.nw
        self.rowPtr = rowPtr
        self.nnz = int(self.rowPtr[-1])
        _lib.check(self._L.rsg_bo_create(C.byref(self._h), C.byref(g), C.byref(f), C.byref(s), self.nrows, self.nw,
                                         C.c_void_p(rowPtr.ctypes.data), C.c_void_p(col.ctypes.data), device))
        del keep

    def close(self):
        if self._h:
            self._L.rsg_bo_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def assemble(self, p, sw, x, state, acc_old, dt: float, add_pos=None, add_val=None, radd_pos=None, radd_val=None):
        """Host vectors in (state: na float64 each, cell states na uint8, old accumulations na*3), J (the pattern's
        nonzeros) and R (nrows) out as numpy arrays; well terms as in assemble_device."""
        p, sw, x, acc = _f64(p), _f64(sw), _f64(x), _f64(acc_old)
        st = np.ascontiguousarray(state, dtype=np.uint8)
        ap = np.ascontiguousarray(add_pos if add_pos is not None else np.zeros(0), dtype=np.int64)
        av = _f64(add_val if add_val is not None else np.zeros(0))
        rp = _i32(radd_pos if radd_pos is not None else np.zeros(0))
        rv = _f64(radd_val if radd_val is not None else np.zeros(0))
        J = np.empty(self.nnz)
        R = np.empty(self.nrows)
        q = lambda a: C.c_void_p(a.ctypes.data) if a.size else None  # noqa: E731
        _lib.check(self._L.rsg_bo_assemble_host(self._h, q(p), q(sw), q(x), q(st), q(acc), float(dt), int(ap.size), q(ap), q(av),
                                                int(rp.size), q(rp), q(rv), q(J), q(R)))
        return J, R

    def assemble_device(self, d_p: int, d_sw: int, d_x: int, d_state: int, d_acc_old: int, dt: float, d_J: int, d_R: int,
                        add_pos=None, add_val=None, radd_pos=None, radd_val=None, stream: int = 0):
        """Device pointers (e.g. torch ``data_ptr()``): state (na float64 each; na uint8), old accumulations (na*3),
        outputs J (the pattern's nonzeros) and R (nrows). Well terms as host arrays (J positions int64, R rows int32)."""
        ap = np.ascontiguousarray(add_pos if add_pos is not None else np.zeros(0), dtype=np.int64)
        av = _f64(add_val if add_val is not None else np.zeros(0))
        rp = _i32(radd_pos if radd_pos is not None else np.zeros(0))
        rv = _f64(radd_val if radd_val is not None else np.zeros(0))
        if ap.size != av.size or rp.size != rv.size:
            raise ValueError("addend positions and values differ in length")
        p = lambda a: C.c_void_p(a.ctypes.data) if a.size else None  # noqa: E731
        _lib.check(self._L.rsg_bo_assemble(self._h, C.c_void_p(d_p), C.c_void_p(d_sw), C.c_void_p(d_x), C.c_void_p(d_state),
                                           C.c_void_p(d_acc_old), float(dt), int(ap.size), p(ap), p(av), int(rp.size), p(rp),
                                           p(rv), C.c_void_p(d_J), C.c_void_p(d_R), C.c_void_p(stream) if stream else None))
