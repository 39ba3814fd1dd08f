import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: takes more than a few seconds")
    # Build the library and the oracles once (a no-op when up to date).
    import __graft_entry__
    __graft_entry__.build()


@pytest.fixture(scope="session")
def golden():
    import numpy as np
    return np.load(Path(__file__).resolve().parent / "golden" / "golden_v1.npz")


@pytest.fixture(scope="session")
def golden_bvh(golden):
    """The small scene's flat arrays from the fixture, as a Bvh."""
    import numpy as np
    from zig_ornament_gb300 import ornament
    textures = []
    for i in golden["scene_texture_map"]:
        data = golden[f"scene_texture_{i}"]
        h, w = data.shape[:2]
        bpc = 1 if data.dtype == np.uint8 else 2
        textures.append(ornament.Texture(data, w, h, 4, bpc, bpc == 2))
    kw = {k[len("scene_"):]: golden[k] for k in golden.files
          if k.startswith("scene_") and k[len("scene_"):] in
          ("tlas_nodes", "blas_nodes", "normals", "normal_indices", "uvs", "uv_indices", "transforms", "materials")}
    return ornament.Bvh.from_arrays(textures=textures, scene_textures_count=int(golden["scene_textures_count"]), **kw)


@pytest.fixture(scope="session")
def golden_camera(golden):
    from zig_ornament_gb300 import _lib
    return _lib.Camera.from_buffer_copy(golden["camera"].tobytes())


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle_lib
    return oracle_lib.Oracle()
