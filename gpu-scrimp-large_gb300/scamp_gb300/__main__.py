"""python -m scamp_gb300: the reference-style command line (see cli.py)."""
from .cli import main

raise SystemExit(main())
