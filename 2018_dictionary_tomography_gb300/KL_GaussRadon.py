"""Moment-matching initial guess of a new atom (KL_GaussRadon.py:57-121).

The reference's ``doKL_ProjGDStep_iso(res, atom, t, R)`` places a new atom by
fitting one Gaussian to the positive part of the residual sinogram (the data
minus the other atoms' projection), iterating:

  1. f = max(0, res) at first, then f = max(0, t res + (1 - t) R(atom));
  2. per angle the mass sum f and the first moments sum f p of f
     (MOM0, MOM1);
  3. the centre M solves  sum_a S0_a (1 - T_a T_a^T) M
                        = sum_a (1 - T_a T_a^T) Ify_a  (orthog_op), where
     Ify_a = sum_i (sum f p_i) w_i(a) is the first moment in world
     coordinates and T_a the projection direction;
  4. the width S^2 = sum f |p - <w, M>|^2 / ((dim - 1) sum f)  (MOM2);
  5. the intensity matches the mass: I = sum f / sum R(atom with I = 1);
until the width, centre and intensity change by at most 1e-4 relative
(at most 100 rounds).  Moments come from the ``gr_sino_moments`` kernel (one
block per angle, FP64, fixed order) over the blended target, which is never
stored; the projection is ``gr_radproj``; the 2 x 2 or 3 x 3 solve is on the
host.

Differences from the reference, stated:
  * the width enters the atom through the kernels' basis exp(-30 m): the
    isotropic and the diagonal r are 1/(sqrt(60) S), so the atom's standard
    deviation is S (the reference's r = S for isotropic and r = 1/S for
    anisotropic atoms predate that basis);
  * the off-diagonal entries of an anisotropic r are set to 0 (the reference
    sets the 2D off-diagonal to 10 and never resets it);
  * the start value is I = 1, x = 0, standard deviation 0.1.
The ``guess`` hook of ``solvers.Newton_linesearch`` takes
``lambda res, atom: doKL_ProjGDStep_iso(res, atom, t, Radon)`` as in the
reference's scripts.
"""
import ctypes

import numpy as np
import torch

from . import _lib, engine

SQRT60 = float(np.sqrt(60.0))


def sino_moments(geom, res, rr=None, t=1.0, scale=1.0):
    """(S0 (A,), S1 (A, kdet), S2 (A, kdet)) FP64 device tensors of
    f = max(0, res) or max(0, t res + (1 - t) scale rr)."""
    dev = geom.device
    A, K = geom.n_angles, geom.kdet
    f64 = dict(dtype=torch.float64, device=dev)
    S0 = torch.empty(A, **f64)
    S1 = torch.empty(A, K, **f64)
    S2 = torch.empty(A, K, **f64)
    st = _lib.load().gr_sino_moments(
        ctypes.byref(geom.struct), res.data_ptr(), None if rr is None else rr.data_ptr(),
        float(t), float(scale), S0.data_ptr(), S1.data_ptr(), S2.data_ptr(),
        ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream))
    _lib.check(st, "gr_sino_moments")
    return S0, S1, S2


def _frames(geom):
    """World-space projection directions T (A, D) and detector axes w (K, A, D)."""
    rec = np.asarray(geom.frames_host, dtype=np.float64)
    K = geom.kdet
    D = K + 1
    T = rec[:, :D]
    w = np.stack([rec[:, D * (1 + k):D * (2 + k)] for k in range(K)])
    return T, w


def moment_fit(res, geom, dim, iso, t=1.0, max_iter=100, rtol=1e-4):
    """(I, x (dim,), r (1 | 3 | 6,)) of the Gaussian whose projection matches
    the moments of max(0, res) (res: float32 device sinogram)."""
    T, w = _frames(geom)
    D = T.shape[1]                       # world dimension of the frames (3 for 2.5D)
    K = w.shape[0]
    pr = 1 if iso else (3 if dim == 2 else 6)
    I, x, S = 1.0, np.zeros(dim), 0.1
    rr, scale = None, 1.0
    proj = torch.empty(geom.shape, dtype=torch.float32, device=geom.device)

    def r_of(S):
        r = np.zeros(pr)
        r[:1 if iso else dim] = 1.0 / (SQRT60 * S)
        return r

    for _ in range(max_iter):
        S0, S1, S2 = (v.cpu().numpy() for v in sino_moments(geom, res, rr, t, scale))
        If = S0.sum()
        if If < 1e-8:
            break                        # no positive residual: keep the current atom
        Ify = np.einsum("ka,kad->ad", S1.T, w)
        op = np.zeros((D, D))
        vec = np.zeros(D)
        for a in range(len(S0)):
            Pa = np.eye(D) - np.outer(T[a], T[a])
            op += S0[a] * Pa
            vec += Pa @ Ify[a]
        try:
            M = np.linalg.solve(op, vec)
        except np.linalg.LinAlgError:
            M = np.zeros(D)
        c = np.einsum("kad,d->ak", w, M)            # <w_i(a), M>
        Ifyy = np.sum(S2 - 2 * c * S1 + c * c * S0[:, None])
        S_new = float(np.sqrt(max(Ifyy, 0.0) / (K * If)))
        x_new = M[:dim]
        r_new = r_of(max(S_new, 1e-12))
        engine.radproj(engine.DeviceAtoms(np.ones(1), x_new.reshape(1, -1),
                                          r_new.reshape(1, -1), geom.device), geom, out=proj)
        mass1 = float(sino_moments(geom, proj)[0].sum().item())
        I_new = If / mass1 if mass1 > 0 else 0.0
        moved = (abs(S - S_new) > rtol * abs(S) or
                 np.linalg.norm(x - x_new) > rtol * np.linalg.norm(x) or
                 abs(I - I_new) > rtol * abs(I))
        I, x, S = I_new, x_new, S_new
        if not moved:
            break
        rr, scale = proj, I
    return I, x, r_of(max(S, 1e-12))


def doKL_ProjGDStep_iso(res, atom, t, R):
    """The reference's guess: ``res`` the residual data - R(atoms incl. this
    one), ``atom`` a one-atom AtomElement (overwritten and returned), ``t``
    the blend weight, ``R`` the GaussTomo operator."""
    geom = R.geometry
    d = res.asarray() if hasattr(res, "asarray") else res
    resd = torch.as_tensor(np.asarray(d) if not isinstance(d, torch.Tensor) else d,
                           dtype=torch.float32).to(geom.device).reshape(geom.shape).contiguous()
    own = engine.radproj(engine.DeviceAtoms(np.asarray(atom.I, dtype=np.float32),
                                            np.asarray(atom.x, dtype=np.float32),
                                            np.asarray(atom.r, dtype=np.float32), geom.device),
                         geom)
    resd = (resd + own).contiguous()     # the residual without this atom
    dim = atom.x.shape[1]
    iso = atom.r.shape[1] == 1
    I, x, r = moment_fit(resd, geom, dim, iso, t)
    atom.I[0] = I
    atom.x[0] = x
    atom.r[0] = r
    return atom
