"""Piecewise-linear time series (TSERIES), restating timeseries.cpp.

TMS_Value (timeseries.cpp:241-263) keeps a cached segment marker between
calls; which segment it interpolates on depends on that marker, and so can the
last bits of a value taken exactly at a knot.  The marker logic is restated as
is, and callers evaluate a series at the same times and in the same order as
the reference's time loop does.
"""


class TimeSeries:
    def __init__(self, times, values):
        if len(times) < 2:
            raise ValueError("Time series size must be greater than one")
        for i in range(1, len(times)):
            if not times[i] > times[i - 1]:
                raise ValueError("Time must increase with index")
        self.points = [(float(t), float(v)) for t, v in zip(times, values)]
        self.size = len(self.points)
        self.marker = 0
        self.value = 0.0

    @classmethod
    def constant(cls, value):
        """TMS_Constant (timeseries.cpp:149-158)."""
        ts = cls.__new__(cls)
        ts.points = []
        ts.size = 0
        ts.marker = 0
        ts.value = float(value)
        return ts

    @classmethod
    def from_file(cls, path):
        """TMS_File (timeseries.cpp:101-147): '#' comments, two numbers per line."""
        t, v = [], []
        with open(path) as f:
            for line in f:
                if line.startswith("#"):
                    continue
                parts = line.split()
                if len(parts) < 2:
                    break
                t.append(float(parts[0]))
                v.append(float(parts[1]))
        if not t:
            raise ValueError("Empty time series file")
        if len(t) == 1:
            ts = cls.__new__(cls)
            ts.points = [(t[0], v[0])]
            ts.size = 1
            ts.marker = 0
            ts.value = 0.0
            return ts
        return cls(t, v)

    def _findmarker(self, time):
        """findmarker (timeseries.cpp:33-57): binary search over [begin, end]."""
        pts = self.points
        low, high = 0, self.size - 1
        while low <= high:
            mid = low + (high - low) // 2
            nxt = pts[mid + 1][0] if mid + 1 < self.size else float("inf")
            if time >= pts[mid][0] and time < nxt:
                return mid
            elif time < pts[mid][0]:
                high = mid - 1
            else:
                low = mid + 1
        return 0

    def __call__(self, time):
        """TMS_Value (timeseries.cpp:241-263)."""
        if self.size == 0:
            return self.value
        pts = self.points
        if time < pts[0][0]:
            return pts[0][1]
        elif time > pts[self.size - 1][0]:
            return pts[self.size - 1][1]
        m = self.marker
        lo = pts[m - 1 if m > 0 else m][0]
        hi = pts[m + 1 if m < self.size - 1 else m][0]
        if time < lo or time > hi:
            self.marker = self._findmarker(time)
        elif time >= lo and m and time < pts[m][0]:
            self.marker = m - 1
        elif m + 1 < self.size and time >= pts[m + 1][0] and time < hi and m < self.size - 1:
            self.marker = m + 1
        m = self.marker
        if m + 1 >= self.size:
            m = self.size - 2
        # linterp (timeseries.cpp:59-64)
        dt = time - pts[m][0]
        return pts[m][1] + (pts[m + 1][1] - pts[m][1]) * (dt / (pts[m + 1][0] - pts[m][0]))
