"""Problem builders: MaxCut (utils/maxcut_helpers.py) and QAP (utils/qap_helpers.py)."""
