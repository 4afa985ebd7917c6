"""Copy a few of the reference's SEP history headers (text) as fixtures.

The reference ships the headers its programs wrote (2d_rtm_restart/Dat/*.H:
a model from create-model-lame.x, receiver gathers from rtm.x, the sponge
filter from abc_init); their binary parts are not in the tree.  They are
copied byte for byte so that the SEP reader is tested on real headers:

    python tests/golden/sep/copy_headers.py
"""
import os
import shutil

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(os.environ.get("REFERENCE_ROOT", "/root/reference"), "2d_rtm_restart", "Dat")
NAMES = ["lambda-layer.H", "seis-Vx-layer.H", "filter.H", "dlambda-layer.H"]

if __name__ == "__main__":
    for n in NAMES:
        shutil.copyfile(os.path.join(SRC, n), os.path.join(HERE, n))
        print("copied", n)
