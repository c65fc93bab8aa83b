"""Restart a coupled flow-rod run from its latest saved files (sopht/utils/restart_sim.py:11-37)."""

from __future__ import annotations

import logging
from pathlib import Path

logger = logging.getLogger(__name__)


def restart_simulation(restart_simulator, io, rod_io, forcing_io, restart_dir: str) -> float:
    """Load the highest-numbered ``sopht_NNNN.h5`` in the working directory into ``io``, the
    matching ``rod_NNNN.h5`` and ``forcing_grid_NNNN.h5`` into ``rod_io`` and ``forcing_io``,
    and the pyelastica state of ``restart_simulator`` from ``restart_dir``; return the time.

    Raises FileNotFoundError when no ``sopht_*.h5`` exists, ValueError when the flow
    and rod times differ.  Flow fields held on the GPU are refilled in place."""
    numbers = [int(p.stem.split("_")[-1]) for p in Path.cwd().glob("sopht_*.h5")]
    if not numbers:
        raise FileNotFoundError("There is no file to load in the directory.")
    latest = max(numbers)
    flow_time = io.load(h5_file_name=f"sopht_{latest:04d}.h5")
    rod_io.load(h5_file_name=f"rod_{latest:04d}.h5")
    forcing_io.load(h5_file_name=f"forcing_grid_{latest:04d}.h5")
    import elastica as ea  # pyelastica owns the rod state files

    rod_time = ea.load_state(restart_simulator, restart_dir, True)
    if flow_time != rod_time:
        raise ValueError("Simulation time of the flow is not matched with the Elastica, check your inputs!")
    logger.info("sopht_%04d.h5 has been loaded", latest)
    return flow_time
