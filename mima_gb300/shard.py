"""Column sharding across ranks (one process per GPU).

Radiation columns are independent (the reference loops over them,
rrtmg_lw_rad.nomcica.f90:453, rrtmg_sw_rad.nomcica.f90:500, and MiMA assigns
latitude bands to MPI ranks, src/atmos_spectral/tools/spec_mpp.f90:42-44), so
a multi-GPU run partitions columns contiguously and needs no collective on the
data path.  Each rank calls the C-ABI on its own slice; outputs are disjoint.
"""
from __future__ import annotations


def column_slice(rank: int, world: int, ncol: int) -> slice:
    """Contiguous, balanced block of columns owned by ``rank``."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    base, extra = divmod(ncol, world)
    start = rank * base + min(rank, extra)
    return slice(start, start + base + (1 if rank < extra else 0))


def env_rank_world():
    import os
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), \
        int(os.environ.get("LOCAL_RANK", "0"))
