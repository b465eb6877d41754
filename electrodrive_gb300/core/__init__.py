"""BEM layer mirroring electrodrive.core (operator, solver, driver, quadrature)."""
