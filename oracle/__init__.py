"""Oracle package: CPU restatement of the reference's CommonNN fit path.

Test infrastructure only; see cnn_oracle.py.
"""
