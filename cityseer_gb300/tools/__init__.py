"""Graph ingest tools: networkx MultiGraph -> NetworkStructure, primal -> dual."""
