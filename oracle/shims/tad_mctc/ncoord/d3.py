from . import cn_d3, cn_d3_gradient  # noqa: F401
