"""Drop-in for stonewall3d/lbm3d.py: same flags, same .npz and checkpoint outputs, sm_103a kernels.

    python lbm3d.py --case p20 --porosity 0.2
"""
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

from stonewall.driver import main  # noqa: E402

if __name__ == "__main__":
    sys.exit(main())
