"""``python -m svierosion_gb300 <command> ...``: the command line interface (svierosion_gb300/cli.py)."""

import sys

from .cli import main

sys.exit(main())
