"""Generate the adjoint golden fixtures: gradients by autograd through the reference.

Usage (needs a checkout of the reference; nothing else in the repository reads it):

    python tests/golden/make_golden_adjoint.py <path to the reference checkout>

For every scene of ``adjoint_scenes.SCENES`` and ``RANDOM_SCENES`` the
reference package runs with
its torch.float64 backend and autograd switched back on (the reference turns
it off at fdtd/backend.py:57-60).  The design object's inverse permittivity is
replaced by a tensor that requires grad (expanded over the three components
for an isotropic Object), the loss is built from cloned field slices after
every ``grid.step()``, and ``loss.backward()`` gives the reference gradient.
Output ``ref_<scene>.npz``: ``design`` (the design tensor), ``loss`` and
``grad`` (d loss / d design), all float64.
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))


def main(ref_path, only=None):
    sys.path.insert(0, HERE)
    sys.path.insert(0, REPO)
    from make_golden import load_reference

    fdtd = load_reference(ref_path)
    import torch

    import adjoint_scenes

    fdtd.set_backend("torch.float64")
    torch.set_grad_enabled(True)
    for name, sc in list(adjoint_scenes.SCENES.items()) + list(adjoint_scenes.RANDOM_SCENES.items()):
        if only and name not in only:
            continue
        grid, obj = sc.build(fdtd)
        p = torch.tensor(sc.design(), dtype=torch.float64, requires_grad=True)
        if p.ndim == 5:
            obj.inverse_permittivity = p
        else:
            obj.inverse_permittivity = p[..., None].expand(*p.shape, 3)
        loss = sc.ref_loss(grid, torch)
        loss.backward()
        np.savez(os.path.join(HERE, f"ref_{name}.npz"), design=p.detach().numpy(), loss=np.array(loss.item()),
                 grad=p.grad.numpy())
        print(name, float(loss), float(np.abs(p.grad.numpy()).max()))


if __name__ == "__main__":
    # optional further arguments: only these scenes
    if len(sys.argv) < 2:
        sys.exit(__doc__)
    main(sys.argv[1], sys.argv[2:] or None)
