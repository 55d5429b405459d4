"""Extract the reference's golden data files into small JSON fixtures.

Run once in a checkout that has the trans_bl reference sources next to it:

    python tests/golden/make_golden.py /path/to/trans_bl

It reads (never modifies) these data files of the reference:
  pre_processing/coefs.bin  -- gfortran sequential unformatted, 20 records of
                               FP64 written by coef_generation.f90:38-57
                               (stretching 1.01, 4 multigrid levels: the level-1
                               penultimate Poisson weights are 2/(1+s), -2/s, 2/(s(1+s)))
  lst_ts/fpp.dat            -- Blasius wall shear per station (main_fs.f90:24-29)
  lst_ts/lst.dat            -- LST growth rate along x (lst_ts/ose_bl.f:81-98)
  lst_ts/saida              -- LST station log: x, Re^(1/2), scaled frequency and
                               the eigenvalue alpha0 per station (ose_bl.f:91)
  lst_ts/ose3d.in           -- the LST starting point (namelist osedata)
and writes coefs_stf1.01_lvl4.json, fpp.json, lst.json and lst_saida.json
beside this script.
"""
import json
import os
import struct
import sys

NAMES = ["record1_stale_fp_fd", "sp_fd", "cp_fd", "pp_fd", "lp_fd",
         "fp_sd", "sp_sd", "cp_sd", "pp_sd", "lp_sd",
         "sp_poi", "cp_poi", "pp_poi", "lp_poi", "w_at_w", "dwydy",
         "sp_integ", "mp_integ", "pp_integ", "lp_integ"]


def read_records(path):
    data = open(path, "rb").read()
    out, off = [], 0
    while off < len(data):
        (n,) = struct.unpack("<i", data[off:off + 4])
        vals = struct.unpack("<%dd" % (n // 8), data[off + 4:off + 4 + n])
        (n2,) = struct.unpack("<i", data[off + 4 + n:off + 8 + n])
        assert n == n2, "record marker mismatch"
        out.append(list(vals))
        off += 8 + n
    return out


def main(ref):
    here = os.path.dirname(os.path.abspath(__file__))
    recs = read_records(os.path.join(ref, "pre_processing", "coefs.bin"))
    assert len(recs) == 20
    json.dump({"stf": 1.01, "lvls": 4, "source": "pre_processing/coefs.bin",
               "records": dict(zip(NAMES, recs))},
              open(os.path.join(here, "coefs_stf1.01_lvl4.json"), "w"), indent=1)
    fpp = [float(l) for l in open(os.path.join(ref, "lst_ts", "fpp.dat")) if l.strip()]
    json.dump({"source": "lst_ts/fpp.dat", "fpp": fpp},
              open(os.path.join(here, "fpp.json"), "w"))
    xs, al = [], []
    for line in open(os.path.join(ref, "lst_ts", "lst.dat")):
        p = line.split()
        if len(p) == 2:
            try:
                xs.append(float(p[0])); al.append(float(p[1]))
            except ValueError:
                pass
    dl = open(os.path.join(ref, "lst_ts", "datalst.dat")).read().split()
    json.dump({"source": "lst_ts/lst.dat", "datalst": dl, "x": xs, "minus_alpha_i_scaled": al},
              open(os.path.join(here, "lst.json"), "w"))
    import re
    num = re.compile(r"[-+]?\d*\.\d+(?:[EeDd][-+]?\d+)?")
    rows = [[float(t.replace("D", "E")) for t in num.findall(l)] for l in open(os.path.join(ref, "lst_ts", "saida"))]
    rows = [r for r in rows if len(r) == 5]
    keep = list(range(0, len(rows), 4)) + ([len(rows) - 1] if (len(rows) - 1) % 4 else [])
    nml = {}
    for line in open(os.path.join(ref, "lst_ts", "ose3d.in")):
        if "=" in line:
            k, v = line.split("=", 1)
            nml[k.strip()] = v.strip().rstrip(",")
    json.dump({"source": "lst_ts/saida, lst_ts/ose3d.in", "stations": len(rows), "dx": rows[1][0] - rows[0][0],
               "osedata": nml, "index": keep, "rows_x_re0_w0_alpha_re_alpha_im": [rows[i] for i in keep]},
              open(os.path.join(here, "lst_saida.json"), "w"))
    print("wrote fixtures to", here)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python make_golden.py <path of the reference checkout>")
    main(sys.argv[1])
