"""
Packed ragged batches and the device pipeline of one GFN-xTB single point.

A batch of molecules of uneven size is packed without padding (offset tables
per molecule for atoms, shells, orbitals and the n^2 / nat^2 / nsh^2 blocks),
uploaded once, and pushed through the CUDA library:

    coordination numbers -> interaction caches -> multipole integrals + H0
    -> persistent SCF (all molecules, one launch) -> analytic gradient.

All device memory is owned by PyTorch (caching allocator); the kernels
allocate nothing. Everything runs on the caller's current CUDA stream.
"""

from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from .params import Tables

F64 = torch.float64


def _prefix(v: np.ndarray) -> np.ndarray:
    out = np.zeros(len(v) + 1, dtype=np.int64)
    np.cumsum(v, out=out[1:])
    return out


def alpha_beta(nel: float, spin: int | None = None) -> tuple[float, float]:
    """
    Alpha/beta electrons (wavefunction/filling.py:180-259): ``spin`` unpaired
    electrons, or the parity of the rounded electron count when None. As in
    the reference, more unpaired electrons than electrons, or a parity that
    does not match the electron count, raise ValueError.
    """
    parity = math.floor(nel + 0.5) % 2
    if spin is None:
        uhf = parity
    else:
        uhf = int(spin)
        if uhf > math.floor(nel + 0.5):
            raise ValueError(f"Number of unpaired electrons ({uhf}) larger than "
                             f"number of electrons ({nel}).")
        if uhf % 2 != parity:
            raise ValueError(f"Odd (even) number of unpaired electrons ({uhf}) but even "
                             f"(odd) number of electrons ({nel}) given.")
    diff = min(uhf, nel)
    nb = (nel - diff) / 2.0
    return nb + diff, nb


class PackedBatch:
    """Device-resident packed layout of a list of molecules."""

    def __init__(self, tables: Tables, numbers: list, positions: list, device=None,
                 charges=None, spins=None):
        device = torch.device(device or "cuda")
        self.device = device
        self.tables = tables
        nums = [np.asarray(n.cpu() if torch.is_tensor(n) else n, dtype=np.int64).ravel() for n in numbers]
        nums = [n[n > 0] for n in nums]
        for n in nums:
            tables.check_elements(n)
        self.nmol = len(nums)
        if self.nmol == 0:
            raise ValueError("empty batch")
        L = tables.i32
        from .params import layout

        lay = layout()
        sh0 = L[lay["DXTB_I_EL_SH0"] : lay["DXTB_I_EL_SH0"] + lay["DXTB_MAXZ"]]
        nshe = L[lay["DXTB_I_EL_NSH"] : lay["DXTB_I_EL_NSH"] + lay["DXTB_MAXZ"]]
        lt = L[lay["DXTB_I_L"] : lay["DXTB_I_L"] + lay["DXTB_MAXSHT"]]
        refocc = tables.f64[lay["DXTB_P_REFOCC"] : lay["DXTB_P_REFOCC"] + lay["DXTB_MAXSHT"]]

        nat = np.array([len(n) for n in nums], dtype=np.int64)
        sh_atom, sh_type, sh_ao, ao_sh, n0 = [], [], [], [], []
        nsh, nao, nel = [], [], []
        for mi, z in enumerate(nums):
            cnt = nshe[z]
            st = np.concatenate([sh0[zz] + np.arange(c) for zz, c in zip(z, cnt)]).astype(np.int32)
            sa = np.repeat(np.arange(len(z), dtype=np.int32), cnt)
            no = 2 * lt[st] + 1
            so = (np.cumsum(no) - no).astype(np.int32)
            aos = np.repeat(np.arange(len(st), dtype=np.int32), no)
            sh_atom.append(sa)
            sh_type.append(st)
            sh_ao.append(so)
            ao_sh.append(aos)
            n0.append(np.repeat(refocc[st] / no, no))
            nsh.append(len(st))
            nao.append(int(no.sum()))
            ch = 0.0 if charges is None else float(charges[mi])
            ne = float(refocc[st].sum()) - ch
            sp = None if spins is None else spins[mi]
            nel.append(alpha_beta(ne, sp))
        nsh = np.array(nsh, dtype=np.int64)
        nao = np.array(nao, dtype=np.int64)
        self.nat, self.nsh, self.nao = nat, nsh, nao
        self.atom_off = _prefix(nat)
        self.shell_off = _prefix(nsh)
        self.ao_off = _prefix(nao)
        self.mat_off = _prefix(nao * nao)
        self.nat2_off = _prefix(nat * nat)
        self.nsh2_off = _prefix(nsh * nsh)
        self.pair_off = _prefix(nsh * (nsh + 1) // 2)
        ws = np.array([_lib.lib().dxtb_scf_workspace_mol(int(n), int(a)) for n, a in zip(nao, nat)])
        self.ws_off = _prefix(ws)

        def dev(a, dt):
            return torch.as_tensor(np.ascontiguousarray(a), dtype=dt).to(device, non_blocking=False)

        self.t = {
            "atom_off": dev(self.atom_off, torch.int64),
            "shell_off": dev(self.shell_off, torch.int64),
            "ao_off": dev(self.ao_off, torch.int64),
            "mat_off": dev(self.mat_off, torch.int64),
            "nat2_off": dev(self.nat2_off, torch.int64),
            "nsh2_off": dev(self.nsh2_off, torch.int64),
            "pair_off": dev(self.pair_off, torch.int64),
            "ws_off": dev(self.ws_off, torch.int64),
            "numbers": dev(np.concatenate(nums), torch.int32),
            "shell_atom": dev(np.concatenate(sh_atom), torch.int32),
            "shell_type": dev(np.concatenate(sh_type), torch.int32),
            "shell_ao": dev(np.concatenate(sh_ao), torch.int32),
            "ao_shell": dev(np.concatenate(ao_sh), torch.int32),
            "n0": dev(np.concatenate(n0), F64),
            "nel": dev(np.array(nel, dtype=np.float64), F64),
            "order": dev(np.argsort(-nao, kind="stable").astype(np.int32), torch.int32),
            "atom_mol": dev(np.repeat(np.arange(self.nmol), nat), torch.int64),
            "par_f": dev(tables.f64, F64),
            "par_i": dev(tables.i32, torch.int32),
        }
        self.numbers = nums
        self.set_positions(positions)

    def set_positions(self, positions: list) -> None:
        pos = [torch.as_tensor(p, dtype=F64).reshape(-1, 3) for p in positions]
        pos = [p[: int(self.nat[i])] for i, p in enumerate(pos)]
        self.positions = torch.cat([p.to(self.device) for p in pos]).contiguous()
        self._struct = None

    def copy_positions_(self, positions) -> None:
        """Overwrite the device positions in place (same molecules), keeping
        their address: a captured ``GraphStep`` reads them from there.
        ``positions``: a list of (nat_m, 3) arrays, or one packed (natoms, 3)
        tensor."""
        if torch.is_tensor(positions) and positions.shape == self.positions.shape:
            self.positions.copy_(positions)
            return
        pos = [torch.as_tensor(p, dtype=F64).reshape(-1, 3)[: int(self.nat[i])].to(self.device)
               for i, p in enumerate(positions)]
        self.positions.copy_(torch.cat(pos))

    @property
    def struct(self) -> _lib.Batch:
        if self._struct is None:
            t = self.t
            self._struct = _lib.Batch(
                self.nmol, int(self.nao.max()), int(self.nat.max()), int(self.nsh.max()),
                t["atom_off"].data_ptr(), t["shell_off"].data_ptr(), t["ao_off"].data_ptr(),
                t["mat_off"].data_ptr(), t["nat2_off"].data_ptr(), t["nsh2_off"].data_ptr(),
                t["pair_off"].data_ptr(), t["numbers"].data_ptr(), self.positions.data_ptr(),
                t["shell_atom"].data_ptr(), t["shell_type"].data_ptr(), t["shell_ao"].data_ptr(),
                t["ao_shell"].data_ptr(),
            )
        return self._struct

    @property
    def total(self) -> dict:
        return {
            "atoms": int(self.atom_off[-1]), "shells": int(self.shell_off[-1]),
            "aos": int(self.ao_off[-1]), "mat": int(self.mat_off[-1]),
            "nat2": int(self.nat2_off[-1]), "nsh2": int(self.nsh2_off[-1]),
            "ws": int(self.ws_off[-1]),
        }


@dataclass
class Result:
    energy: torch.Tensor           # [nmol] total energy (Eh)
    e_scf: torch.Tensor            # [nmol] E_h0 + E_interactions
    e_free: torch.Tensor           # [nmol] -TS
    e_rep: torch.Tensor            # [nmol] repulsion
    iterations: torch.Tensor       # [nmol]
    status: torch.Tensor           # [nmol] int32
    gradient: torch.Tensor | None  # [natoms, 3] packed
    state: dict
    launches: int = 0              # kernels of the library launched by this call


def _seg_sum(values: torch.Tensor, seg: torch.Tensor, nmol: int) -> torch.Tensor:
    """Per-molecule sums of a packed per-atom vector (seg: molecule of each atom, on the device)."""
    return torch.zeros(nmol, dtype=values.dtype, device=values.device).index_add_(0, seg, values)


GB_KERNELS = {"p16": 0, "still": 1}


def scf_launches(L, nmax: int) -> int:
    """Kernels launched by dxtb_scf for a batch whose largest molecule has
    nmax orbitals: one per cluster class up to the largest one present, the
    one-SM launch, the shared-SM launch."""
    thr = (C.c_int32 * 5)()
    _lib.check(L.dxtb_scf_get_size_classes(thr), "size classes")
    cmax = sum(1 for t in thr if nmax >= t)
    return 1 + (1 if cmax >= 1 else 0) + max(0, cmax - 1)


def gb_args(gb: dict) -> tuple:
    """
    (epsilon, kernel, alpb, born_scale, born_offset) of a solvation dict with
    the arguments of ``GeneralizedBorn`` (solvation/alpb.py:213-245):
    ``epsilon`` (dielectric constant), ``alpb`` (default True), ``kernel``
    ("p16" default, or "still"), ``born_scale`` (1.0), ``born_offset`` (0.0).
    """
    eps = float(gb["epsilon"])
    if not eps > 0.0:
        raise ValueError("dielectric constant must be positive")
    kernel = gb.get("kernel", "p16")
    if kernel not in GB_KERNELS:
        raise ValueError(f"unknown Born kernel {kernel!r}")
    return (eps, GB_KERNELS[kernel], 1 if gb.get("alpb", True) else 0,
            float(gb.get("born_scale", 1.0)), float(gb.get("born_offset", 0.0)))


SCF_DEFAULTS = {
    # the reference's ConfigSCF defaults (constants/defaults.py) for the
    # full-mode mixer; the implicit-mode broyden1 uses damp only
    "damp": 0.5, "damp_init": 0.1, "generations": 5, "soft_start": True,
    "diagonal_offset": 0.01, "x_atol_max": 1e-5,
}


def scf_config(maxiter: int, tol: float, scf: dict | None = None) -> _lib.ScfConfig:
    """The C configuration of the SCF. ``scf`` may set ``mixer``
    ("broyden1": implicit mode, "anderson": full mode), ``x_atol``, ``f_atol``,
    ``x_atol_max``, ``damp``, ``damp_init``, ``generations``, ``soft_start``
    and ``diagonal_offset``; ``tol`` is the default of x_atol and f_atol."""
    o = dict(SCF_DEFAULTS)
    o.update(scf or {})
    mixer = o.get("mixer", "broyden1")
    if mixer not in _lib.MIXERS:
        raise ValueError(f"unknown SCF mixer {mixer!r}")
    return _lib.ScfConfig(
        int(maxiter), _lib.MIXERS[mixer], float(o.get("x_atol", tol)), float(o.get("f_atol", tol)),
        float(o["x_atol_max"]), float(o["damp"]), float(o["damp_init"]), int(o["generations"]),
        1 if o["soft_start"] else 0, float(o["diagonal_offset"]),
    )


def run(pb: PackedBatch, *, etemp: float = 300.0, maxiter: int = 250, tol: float = 1e-10,
        forces: bool = False, gb: dict | None = None, state: dict | None = None,
        events: dict | None = None, scf: dict | None = None, collect: bool = True) -> Result:
    """
    One single point for every molecule of the packed batch. With ``events``
    (a dict), CUDA events are recorded on the current stream around each
    stage: events[stage] = (start, end). ``scf`` selects the root solver
    and its tolerances (``scf_config``). With ``collect=False`` only the
    library's kernels are launched (no PyTorch operation allocates) and the
    number of launches is returned; ``collect_result`` then reads the state.
    """
    L = _lib.lib()

    def mark(stage, which):
        if events is not None:
            ev = torch.cuda.Event(enable_timing=True)
            ev.record()
            if which == 0:
                events[stage] = [ev, None]
            else:
                events[stage][1] = ev
    from .data import radii

    tb = pb.tables
    dev = pb.device
    tot = pb.total
    st = _lib.stream_ptr()
    b = C.byref(pb.struct)
    pf, pi = pb.t["par_f"].data_ptr(), pb.t["par_i"].data_ptr()
    s = state if state is not None else {}

    def buf(key, n):
        t = s.get(key)
        if t is None or t.numel() < n:
            t = torch.empty(max(n, 1), dtype=F64, device=dev)
            s[key] = t
        return t

    na, ns, no, nm, n2, g2 = tot["atoms"], tot["shells"], tot["aos"], tot["mat"], tot["nat2"], tot["nsh2"]
    mp = tb.multipole
    cn = buf("cn", na)
    mark("geometry", 0)
    _lib.check(L.dxtb_coordination_number(b, pf, pi, tb.cn_kind, cn.data_ptr(), st), "coordination number")
    launches = 1
    cn_mp = cn
    if mp and tb.cn_kind != 1:
        cn_mp = buf("cn_mp", na)
        _lib.check(L.dxtb_coordination_number(b, pf, pi, 1, cn_mp.data_ptr(), st), "coordination number")
        launches += 1
    gamma, hd = buf("gamma", g2), buf("hd", ns if tb.es3_shell else na)
    erep = buf("erep", na)
    mrad = buf("mrad", na) if mp else None
    sd = buf("sd", 3 * n2) if mp else None
    dd = buf("dd", 9 * n2) if mp else None
    sq = buf("sq", 6 * n2) if mp else None
    _lib.check(
        L.dxtb_interaction_cache(b, pf, pi, cn_mp.data_ptr(), gamma.data_ptr(), hd.data_ptr(),
                                 _lib.ptr(mrad), _lib.ptr(sd), _lib.ptr(dd), _lib.ptr(sq),
                                 erep.data_ptr(), st),
        "interaction cache",
    )
    launches += 1
    gbm = None
    if gb is not None:
        ga = gb_args(gb)
        gbm = buf("gb", n2)
        _lib.check(
            L.dxtb_born_matrix(b, pf, pi, *ga, buf("born", na).data_ptr(), buf("psi", na).data_ptr(),
                               gbm.data_ptr(), st),
            "generalized Born",
        )
        launches += 1
    S, H = buf("S", nm), buf("H", nm)
    D = buf("D", 3 * nm) if mp else None
    Q = buf("Q", 6 * nm) if mp else None
    mark("geometry", 1)
    mark("integrals", 0)
    _lib.check(L.dxtb_multipole_h0(b, pf, pi, cn.data_ptr(), S.data_ptr(), H.data_ptr(),
                                   _lib.ptr(D), _lib.ptr(Q), st), "multipole integrals")
    launches += 1
    mark("integrals", 1)
    P, Cm = buf("P", nm), buf("C", nm)
    W = buf("W", nm) if forces else None
    ev, occ, q = buf("evals", no), buf("occ", no), buf("q", no)
    vorb = buf("vorb", no)
    dp, qp = buf("dp", 3 * na), buf("qp", 6 * na)
    vdp, vqp = buf("vdp", 3 * na), buf("vqp", 6 * na)
    en = buf("energies", 4 * pb.nmol)
    status = s.get("status")
    if status is None or status.numel() < pb.nmol:
        status = torch.empty(pb.nmol, dtype=torch.int32, device=dev)
        s["status"] = status
    ws = buf("ws", tot["ws"])
    kt = etemp * radii.KELVIN2AU
    cfg = scf_config(maxiter, tol, scf)
    scf_args = (b, pf, pi, S.data_ptr(), H.data_ptr(), _lib.ptr(D), _lib.ptr(Q), gamma.data_ptr(),
                hd.data_ptr(), _lib.ptr(sd), _lib.ptr(dd), _lib.ptr(sq), _lib.ptr(gbm),
                pb.t["n0"].data_ptr(), pb.t["nel"].data_ptr(), kt, C.byref(cfg),
                pb.t["ws_off"].data_ptr(), pb.t["order"].data_ptr(), ws.data_ptr(), P.data_ptr(),
                _lib.ptr(W), Cm.data_ptr(), ev.data_ptr(), occ.data_ptr(), q.data_ptr(),
                dp.data_ptr(), qp.data_ptr(), vorb.data_ptr(), vdp.data_ptr(), vqp.data_ptr(),
                en.data_ptr(), status.data_ptr())
    n_scf = scf_launches(L, int(pb.nao.max()))
    grad = None
    if forces:
        # SCF and gradient fused per size class: each class's forces overlap
        # the SCF of the larger classes (grad and dE/dCN zeroed first)
        grad = buf("grad", 3 * na)
        grad.zero_()
        dedcn = buf("dedcn", na)
        dedcn.zero_()
        mark("scf", 0)
        _lib.check(L.dxtb_scf_gradient(*scf_args, cn.data_ptr(), _lib.ptr(mrad), dedcn.data_ptr(),
                                       grad.data_ptr(), st), "SCF and gradient")
        launches += 3 * n_scf  # per class: SCF, pair adjoint, per-molecule terms
        mark("scf", 1)
    else:
        mark("scf", 0)
        _lib.check(L.dxtb_scf(*scf_args, st), "SCF")
        launches += n_scf
        mark("scf", 1)
    if forces:
        mark("gradient", 0)
        if gb is not None:
            _lib.check(
                L.dxtb_born_gradient(b, pf, pi, *ga, q.data_ptr(), s["born"].data_ptr(),
                                     s["psi"].data_ptr(), grad.data_ptr(), st),
                "generalized Born gradient",
            )
            launches += 1
        mark("gradient", 1)
    if not collect:
        return launches
    return collect_result(pb, s, forces, launches)


def collect_result(pb: PackedBatch, s: dict, forces: bool, launches: int = 0) -> Result:
    """The per-molecule results of a single point from its state buffers."""
    na = pb.total["atoms"]
    e4 = s["energies"][: 4 * pb.nmol].view(pb.nmol, 4)
    e_rep = _seg_sum(s["erep"][:na], pb.t["atom_mol"], pb.nmol)
    grad = s["grad"][: 3 * na].view(na, 3) if forces else None
    energy = e4[:, 0] + e4[:, 1] + e_rep
    return Result(energy, e4[:, 0], e4[:, 1], e_rep, e4[:, 2], s["status"][: pb.nmol], grad, s,
                  launches)



class GraphStep:
    """
    The single point of one fixed packed batch as a CUDA graph: the geometry
    kernels, the integrals, the per-class SCF (and gradient) launches on
    their forked streams and the joins, captured once through the library's
    ``dxtb_graph_*`` entry points and replayed for new positions of the same
    molecules (geometry optimisation, molecular dynamics, repeated calls of
    a calculator). The graph keeps the SCF's class priorities as node
    priorities.

    The constructor runs the step once eagerly on a dedicated stream (this
    allocates the state and creates the library's per-stream class streams,
    none of which may happen inside a capture), keeps that result as
    ``first``, and then captures the launches on the same stream.
    ``replay`` copies new positions into the batch's device buffer in place,
    launches the graph and collects the results from the state buffers (a
    few PyTorch reductions, outside the graph). ``run_kw`` are the keyword
    arguments of ``run`` other than ``state``, ``events`` and ``collect``.
    """

    def __init__(self, pb: PackedBatch, **run_kw):
        self.pb = pb
        self.kw = run_kw
        self.state: dict = {}
        self.exec = None
        L = _lib.lib()
        self.stream = torch.cuda.Stream(device=pb.device)
        cur = torch.cuda.current_stream(pb.device)
        self.stream.wait_stream(cur)
        with torch.cuda.stream(self.stream):
            self.first = run(pb, state=self.state, **run_kw)
            self.launches = self.first.launches
            sp = C.c_void_p(self.stream.cuda_stream)
            _lib.check(L.dxtb_graph_begin(sp), "graph capture")
            try:
                run(pb, state=self.state, collect=False, **run_kw)
            finally:
                ex = C.c_void_p()
                rc = L.dxtb_graph_end(sp, C.byref(ex))
            _lib.check(rc, "graph instantiation")
            self.exec = ex
        cur.wait_stream(self.stream)

    def replay(self, positions: list | None = None) -> Result:
        cur = torch.cuda.current_stream(self.pb.device)
        if positions is not None:
            self.pb.copy_positions_(positions)
        self.stream.wait_stream(cur)
        with torch.cuda.stream(self.stream):
            _lib.check(_lib.lib().dxtb_graph_launch(self.exec, C.c_void_p(self.stream.cuda_stream)),
                       "graph launch")
            res = collect_result(self.pb, self.state, bool(self.kw.get("forces", False)), self.launches)
        cur.wait_stream(self.stream)
        return res

    def __del__(self):
        if getattr(self, "exec", None) is not None and _lib is not None:
            try:
                _lib.lib().dxtb_graph_destroy(self.exec)
            except Exception:
                pass
            self.exec = None
