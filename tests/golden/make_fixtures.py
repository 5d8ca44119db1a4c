"""Copy the reference's regression inputs and goldens into tests/golden/.

Run in a checkout next to the Rockable sources:
    python tests/golden/make_fixtures.py /path/to/rockable
The files are the reference's own test data (test/input/* and
test/regression/release/*), gzip-compressed; the tests read them from here
because the reference tree is not available where the GPU tests run.
"""
import gzip
import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))

CASES = {
    "512_particles": ("test/input/512_particles", ["512_particles_bruteforce_LawDefault_noPeriodicity.conf",
                                                    "shape.shp", "drivingSystem.txt"],
                      "test/regression/release/regression_512_particles_LawDefault_noPeriodicity.conf"),
    "518_poly": ("test/input/518_poly", ["518_poly_bruteforce_default_noperiod.conf", "shape.shp",
                                         "drivingSystem.txt"],
                 "test/regression/release/regression_518_poly_default_noperiod.conf"),
    "50_prismes_gravity": ("test/input/50_prismes_gravity", ["50_prismes_gravity.conf", "Shape.shp"],
                           "test/regression/release/regression_50_prismes_gravity.conf"),
}


def main(ref):
    for case, (indir, files, golden) in CASES.items():
        out = os.path.join(HERE, case)
        os.makedirs(out, exist_ok=True)
        for f in files:
            with open(os.path.join(ref, indir, f), "rb") as src, gzip.open(os.path.join(out, f + ".gz"), "wb") as dst:
                shutil.copyfileobj(src, dst)
        with open(os.path.join(ref, golden), "rb") as src, gzip.open(os.path.join(out, "golden.conf.gz"), "wb") as dst:
            shutil.copyfileobj(src, dst)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
