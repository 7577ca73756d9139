"""Test-only stand-in for pandas: DataFrame(list_of_dicts) keeps the rows."""


class DataFrame(list):

    def __init__(self, rows=()):
        super().__init__(rows)

    def __getitem__(self, key):
        if isinstance(key, str):
            return [r[key] for r in self]
        return list.__getitem__(self, key)
