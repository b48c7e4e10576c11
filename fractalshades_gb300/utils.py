"""
Decorators of the model API (same behaviour as the reference's utils.py:
zoom_options, calc_options, interactive_options) and small helpers.
"""
import errno
import functools
import inspect
import os


def mkdir_p(path):
    try:
        os.makedirs(path)
    except OSError as exc:
        if exc.errno == errno.EEXIST and os.path.isdir(path):
            pass
        else:
            raise


def dic_flatten(nested_dic, key_prefix="", sep="@"):
    """Flatten nested dicts: dic[k1]...[kn] becomes flat[k1@...@kn]
    (utils.py:32-45 of the reference)."""
    res = dict()
    if isinstance(nested_dic, dict):
        for key, val in nested_dic.items():
            pre = "" if key_prefix == "" else key_prefix + sep
            res.update(dic_flatten(val, pre + key, sep))
    else:
        res[key_prefix] = nested_dic
    return res


def _store_kwargs(identifier):
    """Decorator for the zoom method: keyword-only call; every argument
    (defaults applied) becomes an instance attribute and the dict is kept as
    ``<identifier>_kwargs`` (utils.py:247-275 of the reference)."""
    def wraps(method):
        @functools.wraps(method)
        def wrapper(self, *args, **kwargs):
            if args:
                raise TypeError(
                    f"{method.__name__} should only accept keyword-arguments ; "
                    f"given positionnal: {args}")
            ba = inspect.signature(method).bind_partial(**kwargs)
            ba.apply_defaults()
            kwargs_dic = dict(ba.arguments)
            setattr(self, identifier + "_kwargs", kwargs_dic)
            for key, val in kwargs_dic.items():
                setattr(self, key, val)
            return method(self, *args, **kwargs)
        return wrapper
    return wraps


class _store_func_name__add_hook:
    """Decorator for the calculation methods: keyword-only call, then the
    calling kwargs and the returned dict are forwarded to
    ``instance.<identifier>_hook(name, kwargs, returned)``
    (utils.py:278-339 of the reference)."""

    def __init__(self, identifier):
        self.identifier = identifier

    def __call__(self, method):
        identifier = self.identifier

        @functools.wraps(method)
        def wrapper(instance, *args, **kwargs):
            if args:
                raise TypeError(
                    f"{method.__name__} should only accept keyword-arguments ; "
                    f"given positionnal: {args}")
            ba = inspect.signature(method).bind_partial(**kwargs)
            ba.apply_defaults()
            kwargs_dic = dict(ba.arguments)
            return_dic = method(instance, *args, **kwargs)
            hook = identifier + "_hook"
            if hasattr(instance, hook):
                getattr(instance, hook)(method.__name__, kwargs_dic, return_dic)

        setattr(wrapper, "_@" + identifier, True)
        return wrapper

    def methods(self, subject):
        tag = "_@" + self.identifier
        return {name: m for name, m in vars(subject).items()
                if callable(m) and hasattr(m, tag)}


class _store_func_name:
    def __init__(self, dic_name):
        self.dic_name = dic_name

    def __call__(self, method):
        @functools.wraps(method)
        def wrapper(*args, **kwargs):
            return method(*args, **kwargs)
        setattr(wrapper, "_@" + self.dic_name, True)
        return wrapper

    def methods(self, subject):
        tag = "_@" + self.dic_name
        return {name: m for name, m in vars(subject).items()
                if callable(m) and hasattr(m, tag)}


zoom_options = _store_kwargs("zoom")
calc_options = _store_func_name__add_hook("calc")
interactive_options = _store_func_name("interactive_options")
