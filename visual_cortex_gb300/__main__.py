"""``python -m visual_cortex_gb300 -c patchV1.cfg [-s seed] [--key value ...]``"""
import sys

from .driver import main

sys.exit(main())
