"""Drop-in ``openSSS.DataReduction``: the span (axial mashing) tables.

``SinogramLUT`` (``Python/openSSS/DataReduction.py:102-172``) and
``SumLORsCounts`` (:174-215) are geometry-time host tables; they live in
``opensss_gb300.geometry`` and are re-exported here under the reference's
module name.
"""

from .geometry import SinogramLUT, SumLORsCounts, expandRings, mashDetectors, span_ring_pairs

__all__ = ["SinogramLUT", "SumLORsCounts", "expandRings", "mashDetectors", "span_ring_pairs"]
