"""Input/output of the synthesis path: atmospheres, line lists, spectra."""
