"""GB300 (sm_103a) online reconstruction for the E906/E1039 spectrometer.

Host-side package over liborgpu.so: layout mirror (layout), C-ABI binding
(_lib), stage pipeline (pipeline), synthetic events (synth).
"""
import os

DATA_DIR = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "data")
GEOMETRY_E906 = os.path.join(DATA_DIR, "basic_geometry_e906.txt")
CALIBRATION_E906 = os.path.join(DATA_DIR, "calibration_e906.txt")
