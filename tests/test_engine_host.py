"""The batched engine's configuration (include/pt_batch.h) is checked on the
host before any device call, so these run without a GPU."""
import pytest

import pathtracer as pt
from pathtracer import abi
from pathtracer.engine import Engine


@pytest.mark.parametrize("fields", [dict(traversal_threads=96), dict(traversal_threads=512),
                                    dict(shade_threads=64), dict(shade_threads=2048), dict(tile_size=300),
                                    dict(wave_paths=1024), dict(precision=1 << 7)])
def test_bad_engine_configurations_are_rejected(fields):
    with pytest.raises(pt.PathTracerError) as err:
        Engine(**fields)
    assert err.value.code == abi.PT_ERR_INVALID_ARG
