"""Data-fit objects (GaussDictCode/transport_loss.py:463-602, KL_GaussRadon.py:52).

``l2_squared_loss(dim)``: value 1/2 sum (x - y)^2 (transport_loss.py:569-585)
and gradient x - y (or y - x for axis=1, :587-602).  ``KL_loss(dim, b)``:
KL(y || x + b) = sum y log(y/(x+b)) - y + (x+b) with 0 log 0 = 0; the
reference's KL_2D (KL_GaussRadon.py:52-54) uses nansum of the same terms with
no background.  Inputs are ProjElements, host arrays or CUDA tensors; values
are computed in float64.  Inside the fitting loops the engine fuses these into
the projection kernel (engine.fit_forward); these classes are the API
surface.
"""
import numpy as np
import torch


def _arr(x):
    if hasattr(x, "asarray"):
        x = x.asarray()
    return x


class Fidelity:
    def __init__(self, dim):
        self.dim = dim

    def __call__(self, x, y):
        return NotImplemented

    def grad(self, x, y, axis=0):
        return NotImplemented


class l2_squared_loss(Fidelity):
    kind = "l2"

    def __call__(self, x, y):
        x, y = _arr(x), _arr(y)
        if isinstance(x, torch.Tensor) or isinstance(y, torch.Tensor):
            x = torch.as_tensor(x)
            y = torch.as_tensor(y, device=x.device)
            d = x.double() - y.double()
            return float(0.5 * torch.sum(d * d).item())
        d = np.asarray(x, dtype=np.float64) - np.asarray(y, dtype=np.float64)
        return 0.5 * float(np.sum(d * d))

    def grad(self, x, y, axis=0):
        x, y = _arr(x), _arr(y)
        return x - y if axis == 0 else y - x


class KL_loss(Fidelity):
    kind = "kl"

    def __init__(self, dim, background=1.0):
        Fidelity.__init__(self, dim)
        if not background > 0:
            raise ValueError("the KL fit needs a positive background")
        self.background = float(background)

    def __call__(self, x, y):
        """KL(y || x + b); x is the model sinogram, y the data."""
        x, y = _arr(x), _arr(y)
        if isinstance(x, torch.Tensor):
            x = x.double().cpu().numpy()
        if isinstance(y, torch.Tensor):
            y = y.double().cpu().numpy()
        g = np.asarray(x, dtype=np.float64) + self.background
        f = np.asarray(y, dtype=np.float64)
        with np.errstate(divide="ignore", invalid="ignore"):
            t = np.where(f > 0, f * np.log(f / g), 0.0)
        return float(np.sum(t - f + g))

    def grad(self, x, y, axis=0):
        x, y = _arr(x), _arr(y)
        return 1.0 - y / (x + self.background)


def KL_2D(f, g):
    """nansum(f (log(f/g) - 1) + g) (KL_GaussRadon.py:52-54)."""
    f = np.asarray(_arr(f), dtype=np.float64)
    g = np.asarray(_arr(g), dtype=np.float64)
    with np.errstate(divide="ignore", invalid="ignore"):
        return float(np.nansum(f * (np.log(f / g) - 1) + g))
