"""Makes the package directory (wnd-charm_gb300/) importable as top-level modules."""
import os
import sys

PKG = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "wnd-charm_gb300")
if PKG not in sys.path:
    sys.path.insert(0, PKG)
