"""Makes tests/golden/part_R256_model.npz from the reference's voxel model
data/part_R256.TopVoxel (read with sgldbench_gb300.topvoxel.read_topvoxel):
the solid mask and the passive mask bit-packed in the file's column-major
voxel order, the fixations and the loads.  The GPU tests cannot read the
reference checkout, so they load this compact copy.

    python tests/golden/make_topvoxel_fixture.py $SGLD_REFERENCE/data/part_R256.TopVoxel
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from sgldbench_gb300 import topvoxel as T  # noqa: E402


def main(src):
    m = T.read_topvoxel(src)
    n = m.nelx * m.nely * m.nelz
    pas = np.zeros(n, dtype=bool)
    pas[m.passive - 1] = True
    np.savez_compressed(
        os.path.join(HERE, "part_R256_model.npz"),
        res=np.array([m.nelx, m.nely, m.nelz], dtype=np.int64),
        solid_bits=np.packbits(m.voxels.reshape(-1, order="F")),
        passive_bits=np.packbits(pas),
        fix_nodes=m.fixing[:, 0].astype(np.int64), fix_flags=m.fixing[:, 1:4].astype(np.int8),
        load_nodes=m.loading[:, 0].astype(np.int64), load_values=m.loading[:, 1:4],
    )


if __name__ == "__main__":
    main(sys.argv[1])
