"""Where the CPU tests find the reference checkout (jrgparkinson/mushy-layer)
whose fixture files they read as data: plotfiles, checkpoints, inputs and
parameter files.

The environment variable MUSHY_LAYER_REFERENCE names the checkout.  Unset,
it defaults to the directory `reference` beside this repository's root.
Tests that read it skip when the file they need is absent (on a machine
without the checkout); the GPU tests never read it.
"""
import os

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DEFAULT = os.path.join(os.path.dirname(ROOT), "reference")


def reference_root():
    return os.environ.get("MUSHY_LAYER_REFERENCE", DEFAULT)


def ref(*parts):
    """Path of a file of the reference checkout."""
    return os.path.join(reference_root(), *parts)
