"""CPU oracle of the lpm-v2 direct sums -- test infrastructure, never the product."""
