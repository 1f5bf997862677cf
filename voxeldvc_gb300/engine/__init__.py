"""Drop-in counterparts of the reference's voxeldvc.engine modules."""
