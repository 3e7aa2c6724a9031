"""Fit records (the reference's ``Record``/``Summary``,
src/cnnclustering/report.py:13-191): one record per fit with the same nine
fields, so code that reads ``Clustering.summary`` keeps working."""
from __future__ import annotations

from collections.abc import MutableSequence


class Record:
    __slots__ = ["n_points", "radius_cutoff", "cnn_cutoff", "member_cutoff", "max_clusters",
                 "n_clusters", "ratio_largest", "ratio_noise", "execution_time"]

    def __init__(self, n_points=None, radius_cutoff=None, cnn_cutoff=None, member_cutoff=None,
                 max_clusters=None, n_clusters=None, ratio_largest=None, ratio_noise=None,
                 execution_time=None):
        for k, v in zip(self.__slots__, (n_points, radius_cutoff, cnn_cutoff, member_cutoff, max_clusters,
                                         n_clusters, ratio_largest, ratio_noise, execution_time)):
            setattr(self, k, v)

    def to_dict(self):
        return {k: getattr(self, k) for k in self.__slots__}

    def __repr__(self):
        attrs = ", ".join(f"{k}={getattr(self, k)!r}" for k in self.__slots__)
        return f"{type(self).__name__}({attrs})"

    def __str__(self):
        cells = ""
        for k in self.__slots__[:-1]:
            v = getattr(self, k)
            if v is None:
                cells += f"{v!r:<10}"
            elif isinstance(v, float):
                cells += f"{v:<10.3f}"
            else:
                cells += f"{v:<10}"
        t = self.execution_time
        if t is not None:
            h, rest = divmod(t, 3600)
            m, s = divmod(rest, 60)
            t = f"{int(h):0>2}:{int(m):0>2}:{s:.3f}"
        header = ("#points   r         c         min       max       #clusters "
                  "%largest  %noise    time     \n")
        return f'{"-" * 95}\n{header}{cells}{t}\n{"-" * 95}\n'


class Summary(MutableSequence):
    def __init__(self, iterable=None):
        self._list = []
        for item in iterable or []:
            self.append(item)

    def __getitem__(self, key):
        return self._list[key]

    def __setitem__(self, key, item):
        if not isinstance(item, Record):
            raise TypeError("Summary can only contain records of type Record")
        self._list[key] = item

    def __delitem__(self, key):
        del self._list[key]

    def __len__(self):
        return len(self._list)

    def __str__(self):
        return self._list.__str__()

    def insert(self, index, item):
        if not isinstance(item, Record):
            raise TypeError("Summary can only contain records of type Record")
        self._list.insert(index, item)
