"""The parity bar of the GPU tests (oracle/parity.py): per path, every
radiance channel within 1e-4 relative (+1e-6 absolute); branch flips counted."""
from oracle.parity import ABS, REL, compare  # noqa: F401
