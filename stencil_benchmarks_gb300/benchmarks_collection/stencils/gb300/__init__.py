from . import basic, horizontal_diffusion, vertical_advection

__all__ = ["basic", "horizontal_diffusion", "vertical_advection"]
