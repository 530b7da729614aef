"""Copies the reference test suite's golden inputs/outputs into tests/golden.

Source: H2P-ERI tests/ (alk32_ccpvdz.mol + D_alk32_ccpvdz.bin -> J_alk32_ccpvdz.bin
used by tests/test_J_input_mat.c; alk26_ccpvdz.mol + D_alk26_ccpvdz.bin ->
K_alk26_ccpvdz.bin used by tests/test_K_input_mat.c). The .bin files are
row-major float64 nbf x nbf matrices (260 x 260 and 210 x 210).
Run where the reference tree is present: python tests/golden/make_golden.py
"""
import os
import shutil

SRC = "/root/reference/tests"
DST = os.path.dirname(os.path.abspath(__file__))
FILES = ["alk32_ccpvdz.mol", "D_alk32_ccpvdz.bin", "J_alk32_ccpvdz.bin",
         "alk26_ccpvdz.mol", "D_alk26_ccpvdz.bin", "K_alk26_ccpvdz.bin"]

if __name__ == "__main__":
    for f in FILES:
        shutil.copyfile(os.path.join(SRC, f), os.path.join(DST, f))
        print("copied", f)
