"""`python -m whatprot_gb300 MODE [VARIANT] [OPTS...]`: the command line."""
import sys

from .cli import main

sys.exit(main())
