from .yaml_loader import build_telescope, load_telescope

__all__ = ["load_telescope", "build_telescope"]
