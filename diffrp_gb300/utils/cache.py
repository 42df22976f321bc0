"""Per-object memoisation used by the render session's lazily evaluated
accessors (semantics of diffrp/utils/cache.py:13-45): ``@cached`` stores a
zero-argument method's result on the instance under the method's qualified
name, ``@key_cached`` under the call argument, ``@singleton_cached`` on the
function object itself."""
import functools

__all__ = ["cached", "key_cached", "singleton_cached", "cache_lookup"]


def cache_lookup(holder, key, compute):
    store = holder.__dict__.setdefault("_cache", {})
    if key not in store:
        store[key] = compute()
    return store[key]


def cached(method):
    name = method.__qualname__

    @functools.wraps(method)
    def wrapper(self):
        return cache_lookup(self, name, lambda: method(self))

    return wrapper


def key_cached(method):
    @functools.wraps(method)
    def wrapper(self, arg):
        return cache_lookup(self, arg, lambda: method(self, arg))

    return wrapper


def singleton_cached(fn):
    name = fn.__qualname__

    @functools.wraps(fn)
    def wrapper():
        return cache_lookup(fn, name, fn)

    return wrapper
