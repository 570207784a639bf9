"""Where the portableRT sources are read from (TEST INFRASTRUCTURE).

The recipes that compile the reference (oracle/Makefile) and the tests that read its
sources or example data take the directory from PRT_REFERENCE_DIR; the default is the
read-only checkout of the development container.  Nothing on a GPU machine needs it:
there the tests that want the sources skip, and the fixtures under tests/golden/ stand in.
"""
import os

REFERENCE_DIR = os.environ.get("PRT_REFERENCE_DIR", "/root/reference")


def reference_path(*parts: str) -> str:
    return os.path.join(REFERENCE_DIR, *parts)
