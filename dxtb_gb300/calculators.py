"""
GFN1/GFN2-xTB calculators with the interface of dxtb's calculators.

``GFN1Calculator(numbers, opts=..., device=..., dtype=...)`` and
``GFN2Calculator`` expose ``get_energy``, ``get_forces``, ``singlepoint``,
``energy``, ``forces`` and ``reset`` like the reference
(calculators/gfn1.py, calculators/gfn2.py:267-298, calculators/types/
abc.py:88-170, types/base.py:758-884). ``numbers`` is 1D for one molecule
or 2D zero-padded for a batch (batch mode 1); positions are Bohr.

Every number comes from the CUDA library (``libdxtb_gb300.so``): integrals,
H0, interactions, the SCF and the analytic gradient. The energy is a
``torch.autograd.Function`` whose backward multiplies the gradient from the
adjoint kernels, so ``energy.backward()`` and ``torch.autograd.grad`` work on
the positions as in the reference.

Not computed (the reference's defaults include it): D3/D4 dispersion;
callers wanting parity pass ``opts={"exclude": ["disp", "d4sc"]}`` to the
reference. The GFN1 halogen-bond term is zero for every accepted element
(its bond strengths are nonzero only for Br, I and At).

SCF options follow the reference's ConfigSCF (constants/defaults.py):
``scf_mode`` "full" (default; the loop of scf/unrolling with the Anderson
mixer, to which the default ``mixer="broyden"`` falls back there, with a
warning, as in scf/unrolling/base.py:80-96) or "implicit" (the xitorch
broyden1 root solver of scf/implicit); ``maxiter`` 100, ``x_atol`` and
``f_atol`` 1e-4, ``x_atol_max`` 1e-5, ``damp`` 0.5, ``damp_init`` 0.1,
``damp_generations`` 5, ``damp_soft_start`` True, ``damp_diagonal_offset``
0.01, ``fermi_etemp`` 300 K. Options the GB300 path does not honour warn or
raise: the EEQ guess (the reference default; the zero-potential SAD start is
used), the linear mixer, SCP modes other than the potential, integral
drivers other than the PyTorch one (the GB300 kernels give its integrals).
"""

from __future__ import annotations

import os
import warnings

import numpy as np
import torch

from . import engine
from .params import Tables

__all__ = ["Calculator", "GFN1Calculator", "GFN2Calculator", "DtypeError", "DeviceError"]


class DtypeError(ValueError):
    """Mismatch of the floating-point type (types/base.py:833-864)."""


class DeviceError(RuntimeError):
    """Mismatch of the device (types/base.py:833-864)."""


class SCFConvergenceError(RuntimeError):
    """SCF did not converge and ``force_convergence`` was requested."""


class SCFConvergenceWarning(UserWarning):
    """SCF did not converge within ``maxiter``."""


# option strings of the reference (constants/labels/scf.py, integrals.py)
_SCF_FULL = ("full", "full_tracking", "unrolling")
_SCF_IMPLICIT = ("default", "implicit")
_MIXER_ANDERSON = ("anderson", "a")
_MIXER_BROYDEN = ("broyden", "b")
_MIXER_LINEAR = ("linear", "l", "simple", "s")
_GUESS_SAD = ("sad", "zero")
_GUESS_EEQ = ("eeq", "equilibration")
_INT_PYTORCH = ("autograd", "pytorch", "torch", "dxtb")
_INT_LIBCINT = ("libcint", "c")
_GRAD_MODES = ("autograd", "backward", "functorch", "row")
# constants/defaults.py
_DEFAULTS = {"maxiter": 100, "x_atol": 1e-4, "f_atol": 1e-4, "x_atol_max": 1e-5, "damp": 0.5,
             "damp_init": 0.1, "damp_generations": 5, "damp_soft_start": True,
             "damp_diagonal_offset": 0.01, "fermi_etemp": 300.0}


def _opt_str(v) -> str:
    return str(v).lower() if not isinstance(v, int) else str(v)


class Result:
    """
    Single-point results with the attribute names of the reference's Result
    (calculators/result.py:36-120). Energies are per molecule (scalars for
    one molecule, (B,) for a batch) where the reference keeps atom-resolved
    tensors; ``cenergies`` holds the repulsion. ``charges``, ``emo`` and
    ``occupation`` are orbital vectors, ``density`` and ``coefficients`` the
    n x n matrices (zero-padded to (B, n, n) for a batch; orbital j is
    column j of ``coefficients``, as in the reference).
    """

    __slots__ = ["charges", "coefficients", "cenergies", "density", "emo", "fenergy", "iter",
                 "occupation", "scf", "total"]

    def get_energies(self) -> dict:
        return {"total": self.total, "scf": self.scf, "fenergy": self.fenergy, **self.cenergies}


_TABLES: dict[str, Tables] = {}


def tables(method: str) -> Tables:
    if method not in _TABLES:
        _TABLES[method] = Tables(method)
    return _TABLES[method]


class _Energy(torch.autograd.Function):
    """Energy with the analytic gradient of the adjoint kernels as backward."""

    @staticmethod
    def forward(ctx, positions, calc, chrg, spin):
        res = calc._run(positions.detach(), chrg, spin, forces=positions.requires_grad)
        ctx.save_for_backward(res["gradient"] if res["gradient"] is not None else torch.empty(0))
        ctx.shape = positions.shape
        return res["energy"].to(positions.dtype)

    @staticmethod
    def backward(ctx, grad_out):
        (g,) = ctx.saved_tensors
        if g.numel() == 0:
            return None, None, None, None
        if grad_out.ndim == 0:
            return grad_out * g, None, None, None
        return grad_out.view(-1, *([1] * (g.ndim - 1))) * g, None, None, None


class Calculator:
    """GFN-xTB single-point calculator on one GB300."""

    method = "gfn2"

    def __init__(self, numbers, par=None, *, classical=None, interaction=None, opts=None,
                 device=None, dtype=None, solvation: dict | None = None):
        if par is not None and isinstance(par, str):
            self.method = par
        if not torch.is_tensor(numbers):
            numbers = torch.as_tensor(numbers)
        if numbers.dtype not in (torch.int16, torch.int32, torch.int64):
            raise DtypeError(f"Atomic numbers must be integers, got {numbers.dtype}")
        # device None: the current CUDA device (this path has no CPU variant)
        self.device = torch.device(device) if device is not None else torch.device("cuda")
        if self.device.type != "cuda":
            raise DeviceError(
                f"the GB300 path runs on a CUDA device only, got device {self.device}"
            )
        self.dtype = dtype or torch.float64
        if self.dtype != torch.float64:
            raise DtypeError("the GB300 path computes in float64 only")
        self.numbers = numbers
        self.batched = numbers.ndim > 1
        self.opts = dict(opts or {})
        self._scf = self._scf_options()
        self.solvation = solvation
        if interaction is not None:
            from .solvation import GeneralizedBorn

            for it in interaction if isinstance(interaction, (list, tuple)) else [interaction]:
                if isinstance(it, GeneralizedBorn):
                    self.solvation = it.as_dict()
                elif isinstance(it, dict) and "epsilon" in it:
                    self.solvation = it
                else:
                    raise NotImplementedError(f"interaction {type(it).__name__} is not on the GB300 path")
        excl = set(self.opts.get("exclude", []))
        # The GFN1 halogen-bond term (components/classicals/halogen/hal.py)
        # needs a halogen with a bond strength: xbond is nonzero only for Br,
        # I and At, outside the elements this path accepts (H-Ar), so it is
        # exactly zero here, as in the reference.
        if "disp" not in excl or (self.method == "gfn2" and "d4sc" not in excl):
            warnings.warn(
                "dispersion is not part of the GB300 path; results equal the reference "
                "with exclude=['disp', 'd4sc']",
                stacklevel=2,
            )
        self.include_rep = "rep" not in excl
        self.tables = tables(self.method)
        nums = numbers.reshape(-1, numbers.shape[-1]).cpu().numpy()
        self._mols = [n[n > 0] for n in nums]
        for n in self._mols:
            self.tables.check_elements(n)
            if self.solvation is not None:
                from .data import radii

                radii.lookup(radii.VDW_D3, n, "van-der-Waals")
        self._pb: engine.PackedBatch | None = None
        self._pb_key = None
        self._graphs: dict = {}  # CUDA graphs of the single point, by ``forces``
        self._state: dict = {}
        self._cache: dict = {}

    # ---- configuration (constants/defaults.py, calculators/config/scf.py) ----
    def _opt(self, key):
        return self.opts.get(key, _DEFAULTS.get(key))

    def _scf_options(self) -> dict:
        """The SCF configuration of ``opts`` (reference defaults where unset),
        with warnings or errors for what the GB300 path does not honour."""
        mode = _opt_str(self.opts.get("scf_mode", "full"))
        mixer = _opt_str(self.opts.get("mixer", "broyden"))
        if mode in _SCF_FULL or mode == "0":
            if mixer in _MIXER_LINEAR or mixer == "0":
                raise NotImplementedError("the linear (simple) mixer is not on the GB300 path")
            if mixer in _MIXER_BROYDEN or mixer == "2":
                # scf/unrolling/base.py:80-96: Broyden falls back to Anderson in full mode
                warnings.warn("Broyden mixer is not implemented for SCF with full gradient "
                              "tracking. Using Anderson mixer instead.", stacklevel=3)
            elif not (mixer in _MIXER_ANDERSON or mixer == "1"):
                raise ValueError(f"Unknown mixer '{mixer}'.")
            kind = "anderson"
        elif mode in _SCF_IMPLICIT or mode == "1":
            kind = "broyden1"  # scf/implicit: xitorch broyden1 whatever the mixer
        else:
            raise NotImplementedError(f"SCF mode '{mode}' is not on the GB300 path")
        scp = _opt_str(self.opts.get("scp_mode", "potential"))
        if scp not in ("potential", "pot", "2"):
            raise NotImplementedError(f"SCP mode '{scp}': the GB300 SCF iterates on the potential")
        guess = _opt_str(self.opts.get("guess", "eeq"))
        if guess in _GUESS_EEQ or guess == "0":
            warnings.warn("the EEQ initial guess is not on the GB300 path; the SAD guess (zero "
                          "charges, zero potential) is used", stacklevel=3)
        elif not (guess in _GUESS_SAD or guess == "1"):
            raise ValueError(f"Unknown guess '{guess}'.")
        drv = _opt_str(self.opts.get("int_driver", "pytorch"))
        if drv in _INT_LIBCINT or drv == "0":
            warnings.warn("the libcint integral driver is not on the GB300 path; the GB300 "
                          "McMurchie-Davidson kernels (equal to the PyTorch driver) are used",
                          stacklevel=3)
        elif not (drv in _INT_PYTORCH or drv == "1"):
            raise ValueError(f"Unknown integral driver '{drv}'.")
        return {
            "mixer": kind,
            "x_atol": float(self._opt("x_atol")),
            "f_atol": float(self._opt("f_atol")),
            "x_atol_max": float(self._opt("x_atol_max")),
            "damp": float(self._opt("damp")),
            "damp_init": float(self._opt("damp_init")),
            "generations": int(self._opt("damp_generations")),
            "soft_start": bool(self._opt("damp_soft_start")),
            "diagonal_offset": float(self._opt("damp_diagonal_offset")),
        }

    @property
    def maxiter(self) -> int:
        return int(self._opt("maxiter"))

    @property
    def etemp(self) -> float:
        return float(self._opt("fermi_etemp"))

    @property
    def tol(self) -> float:
        return self._scf["x_atol"]

    def reset(self) -> None:
        """Forget cached results (types/base.py:758-763)."""
        self._cache.clear()

    def _check(self, positions: torch.Tensor) -> None:
        if positions.dtype != self.dtype:
            raise DtypeError(f"positions have dtype {positions.dtype}, expected {self.dtype}")
        if positions.device.type != "cuda":
            raise DeviceError(f"positions on {positions.device}, expected a CUDA device")

    def _chrg_list(self, chrg, nmol):
        if torch.is_tensor(chrg):
            c = chrg.detach().cpu().reshape(-1).tolist()
        else:
            c = np.atleast_1d(np.asarray(chrg, dtype=np.float64)).tolist()
        return c * nmol if len(c) == 1 else c

    def _run(self, positions, chrg=0.0, spin=None, forces=False):
        """Single point with a one-entry result cache (types/decorators.py:241-288):
        a repeated call with equal positions, charge and spin reuses the last
        result (energy after forces costs nothing)."""
        self._check(positions)
        key = (repr(chrg if not torch.is_tensor(chrg) else chrg.tolist()), repr(spin))
        hit = self._cache.get("last")
        if (hit is not None and hit["key"] == key and (hit["gradient"] is not None or not forces)
                and hit["pos"].shape == positions.shape and torch.equal(hit["pos"], positions)):
            return hit
        out = self._compute(positions, chrg, spin, forces)
        out["key"] = key
        out["pos"] = positions.detach().clone()
        self._cache["last"] = out
        return out

    def _compute(self, positions, chrg=0.0, spin=None, forces=False):
        pos = positions.reshape(-1, positions.shape[-2], 3)
        nmol = len(self._mols)
        chg = self._chrg_list(chrg, nmol)
        spins = None if spin is None else self._chrg_list(spin, nmol)
        key = (tuple(chg), None if spins is None else tuple(spins))
        kw = dict(etemp=self.etemp, maxiter=self.maxiter, tol=self.tol, forces=forces,
                  gb=self.solvation, scf=self._scf)
        if self._pb is None or self._pb_key != key:
            plist = [pos[i, : len(self._mols[i])] for i in range(nmol)]
            self._pb = engine.PackedBatch(self.tables, self._mols, plist, self.device, chg,
                                          [int(s) for s in spins] if spins else None)
            self._pb_key = key
            self._graphs = {}
            # flat index of every real atom in the (nmol * nat_max) layout of
            # the zero-padded input: one gather packs new positions, one
            # scatter unpacks the gradient
            nat_max = pos.shape[-2]
            self._flat = torch.cat([i * nat_max + torch.arange(len(m)) for i, m in
                                    enumerate(self._mols)]).to(self.device)
            from . import autotune

            autotune.ensure(self._pb)  # large batches: the tuned size-class policy
            res = engine.run(self._pb, state=self._state, **kw)
        elif os.environ.get("DXTB_GRAPHS", "1") != "0":
            # the same molecules again (a geometry optimisation, MD, or a
            # repeated call): the second call captures the single point as a
            # CUDA graph, later calls replay it with the new positions
            packed = pos.reshape(-1, 3)[self._flat]
            g = self._graphs.get(forces)
            if g is None and forces not in self._graphs:
                self._pb.copy_positions_(packed)
                try:
                    g = engine.GraphStep(self._pb, **kw)
                    res = g.first
                except RuntimeError as err:
                    # a capture the driver refuses: keep the eager launches
                    warnings.warn(f"CUDA graph capture failed ({err}); launching eagerly",
                                  stacklevel=3)
                    g = None
                    res = engine.run(self._pb, state=self._state, **kw)
                self._graphs[forces] = g
            elif g is None:
                self._pb.copy_positions_(packed)
                res = engine.run(self._pb, state=self._state, **kw)
            else:
                res = g.replay(packed)
        else:
            self._pb.copy_positions_(pos.reshape(-1, 3)[self._flat])
            res = engine.run(self._pb, state=self._state, **kw)
        st = res.status.cpu()
        bad = st[(st != 0)]
        if len(bad):
            codes = set(bad.tolist())
            if codes - {4}:
                from ._lib import STATUS

                raise RuntimeError(f"single point failed: {[STATUS.get(c, c) for c in codes]}")
            if self.opts.get("force_convergence", False):
                raise SCFConvergenceError("SCF did not converge")
            warnings.warn("SCF did not converge within maxiter", SCFConvergenceWarning, stacklevel=3)
        energy = res.energy if self.include_rep else res.energy - res.e_rep
        grad = None
        if forces:
            g = res.gradient
            if not self.include_rep:
                raise NotImplementedError("gradient without repulsion")
            grad = torch.zeros_like(pos).reshape(-1, 3)
            grad[self._flat] = g
            grad = grad.reshape(positions.shape)
        if not self.batched:
            energy = energy[0]
        return {"energy": energy, "gradient": grad, "result": res}

    # ---- public API (calculators/types/abc.py:88-170) ----
    def get_energy(self, positions, chrg=0, spin=None, **_):
        return self.energy(positions, chrg, spin)

    def energy(self, positions, chrg=0, spin=None):
        if positions.requires_grad:
            return _Energy.apply(positions, self, chrg, spin)
        return self._run(positions, chrg, spin)["energy"]

    def get_forces(self, positions, chrg=0, spin=None, grad_mode="autograd", **_):
        """-dE/dR. Every ``grad_mode`` of the reference (autograd, backward,
        functorch, row; calculators/types/autograd.py:146-196) gives the same
        forces here: they come from the adjoint kernels."""
        if grad_mode not in _GRAD_MODES:
            raise ValueError(f"Unknown grad_mode '{grad_mode}'.")
        return self.forces(positions, chrg, spin)

    def forces(self, positions, chrg=0, spin=None):
        r = self._run(positions.detach(), chrg, spin, forces=True)
        return -r["gradient"]

    def hessian(self, positions, chrg=0, spin=None, use_functorch=False,
                derived_quantity="forces", matrix=False, **_):
        """
        Nuclear Hessian (nat, 3, nat, 3), or (3 nat, 3 nat) with ``matrix``
        (calculators/types/autograd.py:198-329). All 6 nat displaced single
        points run as one packed batch with analytic gradients
        (``dxtb_gb300.hessian``); ``use_functorch`` and ``derived_quantity``
        select autodiff variants in the reference and are accepted here. The
        displaced SCFs are converged in implicit mode to min(x_atol, 1e-10).
        """
        if self.batched:
            raise NotImplementedError(
                "Hessian calculation is not supported in batch mode. "
                "Please use the single system mode."
            )
        if derived_quantity not in ("energy", "forces"):
            raise ValueError(f"Unknown derived quantity '{derived_quantity}'.")
        self._check(positions)
        from .hessian import hessian

        spins = None if spin is None else int(spin)
        return hessian(self.tables, self._mols[0], positions.detach(), chrg=float(chrg), spin=spins,
                       etemp=self.etemp, tol=min(self.tol, 1e-10), maxiter=max(self.maxiter, 250),
                       matrix=matrix, device=self.device)

    # ---- properties (calculators/types/autograd.py:331-995) ----
    def dipole(self, positions, chrg=0, spin=None, **_):
        """
        Electric dipole moment (3,) (or (B, 3) batched) in e a0 at the
        converged density: sum_A Z_A R_A - tr(P D0)
        (``calculators/properties/moments/dip.py``), one ``dxtb_dipole_moment``
        launch for the batch. The reference also obtains it as -dE/dF through
        its electric-field interaction; at zero field the two agree (its
        ``test_properties/test_dipole.py`` asserts it).
        """
        from .properties import dipole_moments

        r = self._run(positions.detach(), chrg, spin)
        mu = dipole_moments(self._pb, r["result"].state["P"])
        return mu if self.batched else mu[0]

    dipole_analytical = dipole

    def _hessian_dipole(self, positions, chrg, spin):
        if self.batched:
            raise NotImplementedError(
                "Hessian calculation is not supported in batch mode. "
                "Please use the single system mode."
            )
        self._check(positions)
        from .hessian import hessian

        spins = None if spin is None else int(spin)
        return hessian(self.tables, self._mols[0], positions.detach(), chrg=float(chrg), spin=spins,
                       etemp=self.etemp, tol=min(self.tol, 1e-10), maxiter=max(self.maxiter, 250),
                       device=self.device, dipole_derivative=True)

    def dipole_deriv(self, positions, chrg=0, spin=None, **_):
        """Nuclear dipole derivative d mu / d R, (3, nat, 3) in e, by central
        differences of the dipoles of the displaced single points that also
        give the Hessian (``calculators/types/autograd.py:547-627``)."""
        return self._hessian_dipole(positions, chrg, spin)[1]

    def vibration(self, positions, chrg=0, spin=None, use_functorch=False,
                  project_translational=True, project_rotational=True, **_):
        """Harmonic vibrational analysis (``calculators/types/autograd.py:331-397``):
        ``VibResult`` with frequencies (atomic units; ``use_common_units`` for
        cm^-1) and normal modes (3 nat, nfreqs), from the GPU Hessian."""
        from .properties import vib_analysis

        hess = self.hessian(positions, chrg, spin)
        return vib_analysis(self.numbers, positions, hess,
                            project_translational=project_translational,
                            project_rotational=project_rotational)

    def ir(self, positions, chrg=0, spin=None, use_functorch=False, **_):
        """IR spectrum (``calculators/types/autograd.py:941-993``): ``IRResult``
        with frequencies and intensities (atomic units; ``use_common_units``
        for cm^-1 and km/mol). The Hessian and the dipole derivative come from
        one packed batch of the 6 nat displaced single points."""
        from .properties import IRResult, ir_ints, vib_analysis

        hess, dmu = self._hessian_dipole(positions, chrg, spin)
        vib = vib_analysis(self.numbers, positions, hess)
        return IRResult(vib.freqs, ir_ints(dmu, vib.modes))

    def singlepoint(self, positions, chrg=0, spin=None) -> Result:
        """The single point as a ``Result`` (calculators/types/energy.py:78-414)."""
        r = self._run(positions.detach(), chrg, spin)
        res = r["result"]
        pb = self._pb
        st = res.state
        one = not self.batched

        def per_mol(v):
            return v[0] if one else v

        out = Result()
        out.total = r["energy"]
        out.scf = per_mol(res.e_scf)
        out.fenergy = per_mol(res.e_free)
        out.cenergies = {"repulsion": per_mol(res.e_rep)}
        out.iter = res.iterations.to(torch.int64)
        nmax = int(pb.nao.max())
        vec = {k: torch.zeros(pb.nmol, nmax, dtype=torch.float64, device=pb.device)
               for k in ("q", "evals", "occ")}
        mat = {k: torch.zeros(pb.nmol, nmax, nmax, dtype=torch.float64, device=pb.device)
               for k in ("P", "C")}
        for i in range(pb.nmol):
            n, o0, m0 = int(pb.nao[i]), int(pb.ao_off[i]), int(pb.mat_off[i])
            for k in vec:
                vec[k][i, :n] = st[k][o0 : o0 + n]
            order = torch.argsort(vec["evals"][i, :n])
            vec["evals"][i, :n] = vec["evals"][i, :n][order]
            vec["occ"][i, :n] = vec["occ"][i, :n][order]
            mat["P"][i, :n, :n] = st["P"][m0 : m0 + n * n].view(n, n)
            # rows of the C block are orbitals (unsorted); columns here
            mat["C"][i, :n, :n] = st["C"][m0 : m0 + n * n].view(n, n)[order].T
        out.charges = per_mol(vec["q"])
        out.emo = per_mol(vec["evals"])
        out.occupation = per_mol(vec["occ"])
        out.density = per_mol(mat["P"])
        out.coefficients = per_mol(mat["C"])
        return out


class GFN1Calculator(Calculator):
    """GFN1-xTB (calculators/gfn1.py)."""

    method = "gfn1"


class GFN2Calculator(Calculator):
    """GFN2-xTB (calculators/gfn2.py:267-298)."""

    method = "gfn2"
