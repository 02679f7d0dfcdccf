"""Graph colouring enums (reference: graph/Enums.h:20-33, bound as pbat.graph)."""

import enum


class GreedyColorOrderingStrategy(enum.IntEnum):
    Natural = 0
    SmallestDegree = 1
    LargestDegree = 2


class GreedyColorSelectionStrategy(enum.IntEnum):
    LeastUsed = 0
    FirstAvailable = 1
