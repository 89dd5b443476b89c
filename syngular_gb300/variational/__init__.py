"""Device-side building blocks of the reference's variational package
(``variational/dmrg.py``): the DMRG environment blocks and the two-site
effective contraction.  The Lanczos optimiser and the sweep driver around
them are not part of this library."""
from .dmrg import DMRG

__all__ = ["DMRG"]
