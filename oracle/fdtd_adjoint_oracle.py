"""CPU oracle of the reverse-time adjoint: numpy float64, stage by stage.

TEST INFRASTRUCTURE ONLY.  Only ``tests/`` may import this module, as the
checker of the GPU adjoint.  The product path never imports it.

The reference has no adjoint; its gradients come from autograd through its
torch backend (the fixtures ``tests/golden/ref_adj_*.npz`` hold such
gradients, made by ``tests/golden/make_golden_adjoint.py``).  This module
restates the same gradient as explicit transposes of the stages of
``fdtd_oracle.Grid.update_E`` / ``update_H`` (which follow
fdtd/grid.py:275-325), applied in reverse order:

* curl_H / curl_E (fdtd/grid.py:29-76): transposes of the dropped-edge
  one-sided differences;
* bulk updates E += c eps^-1 curl_H, H -= c mu^-1 curl_E;
* PML auxiliaries and corrections (fdtd/boundaries.py:409-487, compact
  storage of ``fdtd_oracle.PML``);
* periodic copies (fdtd/boundaries.py:184-219): F[dst] = F[src] transposes to
  lam[src] += lam[dst], lam[dst] = 0 (on an axis of one plane the copy and its
  transpose are the identity);
* objects (fdtd/objects.py:118-277), including the gradient with respect to a
  design object's inverse permittivity;
* hard sources (fdtd/sources.py:476-486) zero the adjoint at their cells; soft
  sources do nothing;
* detector samples add the loss gradient (the seeds).

``tests/test_adjoint_oracle.py`` pins this restatement to the fixtures and to
central differences of the oracle forward on random scenes.
"""

import numpy as np

from oracle import fdtd_oracle as fo


def _diff_bwd_T(v, axis):
    """Transpose of fdtd_oracle._diff_bwd (a[n] - a[n-1], first plane 0)."""
    out = np.zeros_like(v)
    n = v.shape[axis]
    hi = [slice(None)] * v.ndim
    lo = [slice(None)] * v.ndim
    hi[axis] = slice(1, n)
    lo[axis] = slice(0, n - 1)
    out[tuple(hi)] += v[tuple(hi)]
    out[tuple(lo)] -= v[tuple(hi)]
    return out


def _diff_fwd_T(v, axis):
    """Transpose of fdtd_oracle._diff_fwd (a[n+1] - a[n], last plane 0)."""
    out = np.zeros_like(v)
    n = v.shape[axis]
    hi = [slice(None)] * v.ndim
    lo = [slice(None)] * v.ndim
    hi[axis] = slice(1, n)
    lo[axis] = slice(0, n - 1)
    out[tuple(hi)] += v[tuple(lo)]
    out[tuple(lo)] -= v[tuple(lo)]
    return out


def curl_H_T(w):
    """lam_H contribution of a curl_H output adjoint ``w``."""
    out = np.zeros_like(w)
    out[..., 2] += _diff_bwd_T(w[..., 0], 1) - _diff_bwd_T(w[..., 1], 0)
    out[..., 1] += -_diff_bwd_T(w[..., 0], 2) + _diff_bwd_T(w[..., 2], 0)
    out[..., 0] += _diff_bwd_T(w[..., 1], 2) - _diff_bwd_T(w[..., 2], 1)
    return out


def curl_E_T(w):
    """lam_E contribution of a curl_E output adjoint ``w``."""
    out = np.zeros_like(w)
    out[..., 2] += _diff_fwd_T(w[..., 0], 1) - _diff_fwd_T(w[..., 1], 0)
    out[..., 1] += -_diff_fwd_T(w[..., 0], 2) + _diff_fwd_T(w[..., 2], 0)
    out[..., 0] += _diff_fwd_T(w[..., 1], 2) - _diff_fwd_T(w[..., 2], 1)
    return out


def _slab_inner(pml, side):
    """Index of the slab-local planes where the auxiliary increment applies."""
    inner = [slice(None)] * 3
    inner[pml.axis] = slice(1, None) if side == "E" else slice(None, -1)
    return tuple(inner)


def _psi_update_T(pml, side, mu, lam_slab):
    """Transpose of PML.phi_E / phi_H for adjoint auxiliaries ``mu`` (2, slab):
    adds to lam_slab (the field adjoint on the slab) and scales mu by b."""
    n, t1, t2 = pml.axis, (pml.axis + 1) % 3, (pml.axis + 2) % 3
    b = pml._prof(pml.bE if side == "E" else pml.bH)
    c = pml._prof(pml.cE if side == "E" else pml.cH)
    inner = _slab_inner(pml, side)
    diff_T = _diff_bwd_T if side == "E" else _diff_fwd_T
    for q, comp in ((0, t2), (1, t1)):
        v = np.zeros(pml.slab_shape)
        v[inner] = (mu[q] * c)[inner]
        lam_slab[..., comp] += diff_T(v, n)
    mu *= b


def _correct_T(pml, side, mu, lam):
    """Transpose of PML.correct_E / correct_H: mu += dF/dpsi^T lam."""
    t1, t2 = (pml.axis + 1) % 3, (pml.axis + 2) % 3
    loc = pml._loc()
    g = pml.grid
    if side == "E":
        ce = g.courant_number * g.inverse_permittivity[loc]
        mu[0] += -ce[..., t1] * lam[loc + (t1,)]
        mu[1] += ce[..., t2] * lam[loc + (t2,)]
    else:
        cm = g.courant_number * g.inverse_permeability[loc]
        mu[0] += cm[..., t1] * lam[loc + (t1,)]
        mu[1] += -cm[..., t2] * lam[loc + (t2,)]


def _periodic_T(bnd, side, lam):
    if lam.shape[bnd.axis] <= 1:
        return  # the copy of a one-plane axis is the identity, and so is its transpose
    if side == "E":  # E[0] = E[-1]
        lam[bnd._plane(-1)] += lam[bnd._plane(0)]
        lam[bnd._plane(0)] = 0.0
    else:  # H[-1] = H[0]
        lam[bnd._plane(0)] += lam[bnd._plane(-1)]
        lam[bnd._plane(-1)] = 0.0


def _source_T(src, side, lam):
    if isinstance(src, fo.PlaneSource):
        comp = src._Epol if side == "E" else src._Hpol
        lam[src.x, src.y, src.z, comp] = 0.0


def _detector_cells(det):
    """Index tuple of the cells a detector samples, in record order."""
    if isinstance(det, (fo.PlaneDetector, fo.DFTPlaneDetector)):
        return (det.x, det.y, det.z)
    if isinstance(det, fo.BlockDetector):
        xs, ys, zs = np.meshgrid(det.x, det.y, det.z, indexing="ij")
        return (xs, ys, zs)
    return (np.asarray(det.x), np.asarray(det.y), np.asarray(det.z))


def forward_records(grid, steps, design):
    """Run ``steps`` steps of an oracle grid; return the detector records
    (per detector name: {"E": (steps, ...), "H": ...} or {"dft": ...}) and
    the design-box curls (steps, box, 3) captured before every E half."""
    curls = []
    for _ in range(steps):
        curls.append(fo.curl_H(grid.H)[design._loc()].copy())
        grid.step()
    recs = {}
    for det in grid.detectors:
        if isinstance(det, fo.DFTPlaneDetector):
            recs[det.name] = {"dft": det.dft.copy()}
        else:
            recs[det.name] = {"E": np.stack(det.E[-steps:]), "H": np.stack(det.H[-steps:])}
    return recs, np.stack(curls)


def adjoint_gradient(grid, steps, design, q0, seeds, curls):
    """Gradient of a loss with respect to ``design.inverse_permittivity``.

    ``grid`` is the oracle grid after the forward run (its components define
    the transposed stages), ``q0`` the step index the run started at,
    ``seeds`` per detector name {"E"/"H": dL/d records (steps, ...)} or
    {"dft": dL/d dft as complex (re + i im)}, ``curls`` from
    ``forward_records``.  Returns an array shaped like the design's inverse
    permittivity."""
    g = grid
    lamE = np.zeros_like(g.E)
    lamH = np.zeros_like(g.H)
    muE = {id(b): np.zeros((2,) + b.slab_shape) for b in g.boundaries if isinstance(b, fo.PML)}
    muH = {id(b): np.zeros((2,) + b.slab_shape) for b in g.boundaries if isinstance(b, fo.PML)}
    grad = np.zeros_like(design.inverse_permittivity)
    c = g.courant_number
    for t in range(steps - 1, -1, -1):
        q = q0 + t
        # --- transposed H half
        for det in g.detectors:
            s = seeds.get(det.name, {})
            if s.get("H") is not None:
                np.add.at(lamH, _detector_cells(det), s["H"][t])
        for src in reversed(g.sources):
            _source_T(src, "H", lamH)
        for b in reversed(g.boundaries):
            if isinstance(b, fo.PML):
                _correct_T(b, "H", muH[id(b)], lamH)
            else:
                _periodic_T(b, "H", lamH)
        lamE += curl_E_T(-c * g.inverse_permeability * lamH)
        for b in reversed(g.boundaries):
            if isinstance(b, fo.PML):
                sl = np.zeros(b.slab_shape + (3,))
                _psi_update_T(b, "H", muH[id(b)], sl)
                lamE[b._loc()] += sl
        # --- transposed E half
        for det in g.detectors:
            s = seeds.get(det.name, {})
            if s.get("E") is not None:
                np.add.at(lamE, _detector_cells(det), s["E"][t])
            if s.get("dft") is not None:
                box = _detector_cells(det)
                for f, fr in enumerate(det.frequencies):
                    cs, sn = fo.dft_factor(fr, q, g.time_step)
                    lamE[box] += s["dft"][f].real * cs + s["dft"][f].imag * sn
        for src in reversed(g.sources):
            _source_T(src, "E", lamE)
        for b in reversed(g.boundaries):
            if isinstance(b, fo.PML):
                _correct_T(b, "E", muE[id(b)], lamE)
            else:
                _periodic_T(b, "E", lamE)
        lam_curl = np.zeros_like(lamE)
        for o in reversed(g.objects):
            loc = o._loc()
            lam = lamE[loc]
            if isinstance(o, fo.AbsorbingObject):
                f = o.absorption_factor
                lam_curl[loc] += c * o.inverse_permittivity / (1 + f) * lam
                lamE[loc] = lam * ((1 - f) / (1 + f))
            elif isinstance(o, fo.AnisotropicObject):
                lam_curl[loc] += c * np.einsum("xyzab,xyza->xyzb", o.inverse_permittivity, lam)
                if o is design:
                    grad += c * np.einsum("xyza,xyzb->xyzab", lam, curls[t])
            else:
                lam_curl[loc] += c * o.inverse_permittivity * lam
                if o is design:
                    grad += c * curls[t] * lam
        lam_curl += c * g.inverse_permittivity * lamE
        lamH += curl_H_T(lam_curl)
        for b in reversed(g.boundaries):
            if isinstance(b, fo.PML):
                sl = np.zeros(b.slab_shape + (3,))
                _psi_update_T(b, "E", muE[id(b)], sl)
                lamH[b._loc()] += sl
    return grad
