"""Where the fixture generators find the sdepy checkout they run.

The path is the generator's first argument, else the SDEPY_REFERENCE
environment variable; there is no default, so a generator never runs a
checkout its caller did not name."""
import os
import sys


def reference_dir(argv=None):
    argv = sys.argv if argv is None else argv
    if len(argv) > 1 and argv[1]:
        return argv[1]
    env = os.environ.get('SDEPY_REFERENCE')
    if env:
        return env
    sys.exit('usage: {} REFERENCE_DIR [...]  (or set SDEPY_REFERENCE to the '
             'sdepy checkout)'.format(os.path.basename(argv[0])))
