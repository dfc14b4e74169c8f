#!/bin/sh
# Regenerates the golden fixtures in tests/golden/ from MD-Lab's own _nocl
# build.  Needs the MD-Lab source tree: REF_DIR or MDLAB_SRC, else this
# container's read-only mount of it; the fixtures it writes are committed, so
# the tests themselves never need it.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
ROOT=$(cd "$HERE/../.." && pwd)
REF_DIR=${REF_DIR:-${MDLAB_SRC:-/root/reference}}
if [ ! -f "$REF_DIR/md_pimd_x.c" ]; then
  echo "make_golden.sh: no MD-Lab source tree at '$REF_DIR' (set MDLAB_SRC)" >&2
  exit 2
fi
make -s -C "$ROOT/oracle" ref REF_DIR="$REF_DIR"
OUT=$ROOT/oracle/_ref
for v in d3l8 d3l4 d2l4; do
  gcc -O2 -ffp-contract=off -w -I "$OUT/src_$v" -o "$OUT/make_golden_$v" "$HERE/make_golden.c" \
      -L "$OUT" -lxmd_x_$v -Wl,-rpath,"$OUT" -lm
done
G3="$OUT/make_golden_d3l4"
G38="$OUT/make_golden_d3l8"
G2="$OUT/make_golden_d2l4"
cd "$HERE"
# 2D harmonic trap, N=4 bosons, P=32, beta=2, V=2 exp(-r^2/0.25), dt=0.01
$G2 pimd d2l4_cfg1.bin N=4 P=32 vi=1 beta=2 g=1.5707963267948966 s=0.5 dt=0.01 seed=2024 steps=1000 every=100
# 3D trap, V=3 exp(-r^2/0.25), beta=4, dt=0.005, three statistics
$G3 pimd d3l4_trap_vi1.bin N=8 P=8 vi=1 beta=4 seed=11 steps=1000 every=100
$G3 pimd d3l4_trap_vi05.bin N=8 P=8 vi=0.5 beta=4 seed=12 steps=200 every=50
$G3 pimd d3l4_trap_vi0.bin N=8 P=8 vi=0 beta=4 seed=13 steps=200 every=50
# ragged sizes, P=2 (no interior beads), N=1, grouped chains (f=3, fc=3)
$G3 pimd d3l4_trap_n37p6.bin N=37 P=6 vi=0.75 beta=3 seed=14 steps=20 every=10
$G3 pimd d3l4_trap_p2.bin N=5 P=2 vi=1 beta=2 seed=15 steps=50 every=25
$G3 pimd d3l4_trap_n1.bin N=1 P=8 vi=1 beta=4 seed=16 steps=50 every=25
$G3 pimd d3l4_trap_chain3.bin N=6 P=4 vi=0.25 beta=4 f=3 fc=3 seed=17 steps=50 every=25
# periodic electron gas with Ewald (alpha = 5.6/L), minimum-image springs, wrap
$G3 pimd d3l4_ueg.bin N=8 P=4 vi=0.6 rs=2 theta=0.5 ueg=1 image=1 pbc=1 nsum=3 dt=0.05 seed=18 steps=20 every=10
# the reference's default chain length
$G38 pimd d3l8_trap.bin N=6 P=8 vi=1 beta=4 seed=19 steps=100 every=50
# cubic vs quadratic exchange paths
$G3 cubic d3l4_cubic.bin N=7 P=5 vi=0.5 beta=2 seed=21 image=0
$G3 cubic d3l4_cubic_img.bin N=6 P=4 vi=1 beta=3 seed=22 image=1 box=2.5
# two species: unpolarised electron gas (5 up + 4 down, Ewald) and two
# trapped species of different mass with Gaussian interactions
$G3 two d3l4_two_ueg.bin N=5 Nb=4 P=4 vi=0.8 rs=2 theta=0.5 ueg=1 image=1 pbc=1 nsum=3 dt=0.05 seed=23 steps=10 mb=1
$G3 two d3l4_two_trap.bin N=6 Nb=5 P=4 vi=0.5 beta=3 seed=24 steps=20 mb=2
$G2 two d2l4_two_trap.bin N=3 Nb=7 P=6 vi=1 beta=2 seed=25 steps=20 mb=0.5
# observables outside the step (plain and centroid virial, g(r), polymer wrap,
# function-valued accumulators) after a trajectory without the per-step wrap
$G3 obs d3l4_obs_ueg.bin N=9 P=6 vi=0.7 rs=2 theta=0.5 ueg=1 image=1 nsum=2 dt=0.05 seed=31 steps=15
$G2 obs d2l4_obs_trap.bin N=7 P=5 vi=1 beta=3 seed=32 steps=10 box=3
# random numbers and isolated pair callbacks
$G3 rng rng.bin
$G3 pairs d3_pairs.bin
$G2 pairs d2_pairs.bin
ls -la "$HERE"/*.bin
