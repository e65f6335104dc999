"""Drop-in counterpart of the reference package of the same name."""
