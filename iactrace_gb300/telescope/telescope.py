"""The Telescope (telescope/telescope.py of the reference)."""
from __future__ import annotations

from ..core.render import render, render_debug


class Telescope:
    """telescope/telescope.py:22-236: mirror groups, obstruction groups, sensors.

    Instances are treated as immutable: the editors in ``operations`` return
    new telescopes, and packed device tables are cached per instance.
    """

    def __init__(self, mirror_groups, obstruction_groups=None, sensors=None, name: str = "telescope"):
        self.mirror_groups = list(mirror_groups)
        self.obstruction_groups = obstruction_groups
        self.sensors = list(sensors) if sensors else []
        self.name = name

    def __call__(self, sources, values, source_type="point", sensor_idx: int = 0, debug: bool = False, seed: int = 0):
        """telescope/telescope.py:56-83 (seed: jitter stream of 'extended' sources)."""
        if debug:
            return render_debug(self, sources, values, source_type, sensor_idx, seed=seed)
        return render(self, sources, values, source_type, sensor_idx, seed=seed)

    def __getstate__(self):
        st = dict(self.__dict__)
        st.pop("_packed", None)
        st.pop("_stages", None)
        return st

    @classmethod
    def from_yaml(cls, filename, integrator, key=None) -> "Telescope":
        from ..io.yaml_loader import load_telescope
        return load_telescope(filename, integrator, key)

    # convenience editors (telescope/telescope.py:100-236)
    def resample_mirrors(self, integrator, key):
        from . import operations as o
        return o.resample_mirrors(self, integrator, key)

    def set_mirror_positions(self, group_idx, positions):
        from . import operations as o
        return o.set_mirror_positions(self, group_idx, positions)

    def set_mirror_rotations(self, group_idx, rotations):
        from . import operations as o
        return o.set_mirror_rotations(self, group_idx, rotations)

    def scale_mirror_weights(self, group_idx, scale_factors):
        from . import operations as o
        return o.scale_mirror_weights(self, group_idx, scale_factors)

    def apply_roughness(self, roughness_arcsec):
        from . import operations as o
        return o.apply_roughness(self, roughness_arcsec)

    def apply_roughness_to_group(self, group_idx, roughness):
        from . import operations as o
        return o.apply_roughness_to_group(self, group_idx, roughness)

    def apply_misalignment_to_group(self, group_idx, sigma_h, sigma_v, key):
        from . import operations as o
        return o.apply_misalignment_to_group(self, group_idx, sigma_h, sigma_v, key)

    def apply_displacement_to_group(self, group_idx, sigma_z, key):
        from . import operations as o
        return o.apply_displacement_to_group(self, group_idx, sigma_z, key)

    def get_mirrors_by_stage(self, stage):
        from . import operations as o
        return o.get_mirrors_by_stage(self, stage)

    def get_mirror_count(self):
        from . import operations as o
        return o.get_mirror_count(self)

    def add_sensor(self, sensor):
        from . import operations as o
        return o.add_sensor(self, sensor)

    def replace_sensor(self, sensor, idx=0):
        from . import operations as o
        return o.replace_sensor(self, sensor, idx)

    def remove_sensor(self, idx=0):
        from . import operations as o
        return o.remove_sensor(self, idx)

    def set_sensor_position(self, idx, position):
        from . import operations as o
        return o.set_sensor_position(self, idx, position)

    def set_sensor_rotation(self, idx, rotation):
        from . import operations as o
        return o.set_sensor_rotation(self, idx, rotation)

    def focus(self, delta_z, sensor_idx=0):
        from . import operations as o
        return o.focus(self, delta_z, sensor_idx)

    def get_sensor_count(self):
        from . import operations as o
        return o.get_sensor_count(self)

    def add_obstruction(self, obstruction):
        from . import operations as o
        return o.add_obstruction(self, obstruction)

    def remove_obstruction(self, group_idx):
        from . import operations as o
        return o.remove_obstruction(self, group_idx)

    def clear_obstructions(self):
        from . import operations as o
        return o.clear_obstructions(self)

    def get_obstruction_count(self):
        from . import operations as o
        return o.get_obstruction_count(self)

    def clone(self):
        from . import operations as o
        return o.clone(self)

    def get_info(self):
        from . import operations as o
        return o.get_info(self)
