"""python -m cyrsoxs_gb300 <morphology.h5> [HDF5 output directory]"""
import sys

from .cli import main

sys.exit(main())
