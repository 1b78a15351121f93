from . import cn_d4  # noqa: F401
