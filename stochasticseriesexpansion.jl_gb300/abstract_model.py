"""Model plugin interface (restatement of src/abstract_model.jl:17-54).

A model is constructed from a parameter dict and must provide

* ``generate_sse_data()``        -> :class:`SSEData` (bond graph + vertex tables)
* ``get_opstring_estimators()``  -> list of :class:`MagnetizationEstimatorSpec`
* ``leg_count()`` (classmethod)  -> maximum legs per bond operator (4 for two-site bonds)
* ``normalization_site_count()`` -> number of physical sites used to normalise observables
* ``magnetization_state(site, state)`` when magnetisation estimators are requested
"""

from __future__ import annotations


class AbstractModel:
    @classmethod
    def leg_count(cls) -> int:
        raise NotImplementedError

    def generate_sse_data(self):
        raise NotImplementedError

    def get_opstring_estimators(self):
        return []

    def normalization_site_count(self) -> int:
        raise NotImplementedError

    def magnetization_state(self, site_idx: int, state_idx: int) -> float:
        raise NotImplementedError
