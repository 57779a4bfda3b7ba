"""pytest plugin used only by make_golden.py when it runs the reference's own
unit tests: restores ``np.complex`` and the ``newshape=`` keyword of
``np.reshape``, both of which the reference uses and NumPy 2 removed."""
import numpy as np

if not hasattr(np, "complex"):
    np.complex = complex

_orig_reshape = np.reshape


def _reshape(a, *args, **kw):
    if "newshape" in kw:
        kw["shape"] = kw.pop("newshape")
    return _orig_reshape(a, *args, **kw)


np.reshape = _reshape
