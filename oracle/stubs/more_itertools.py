"""Test-only stand-in for the two more_itertools helpers the reference uses."""


def flatten(it):
    for x in it:
        for y in x:
            yield y


def distribute(n, iterable):
    items = list(iterable)
    return [items[i::n] for i in range(n)]
