#!/usr/bin/env python3
"""Drop-in for the reference's grad.py: `python grad.py algo=<cg|sd|LBFGS> eps...` in the code
directory (master.py:21, 212-224)."""
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))))
from sparc_flows_gb300.gradient import main  # noqa: E402

sys.exit(main())
