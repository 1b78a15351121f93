def get_zvalence(*args, **kwargs):
    raise NotImplementedError
