#!/usr/bin/env bash
# Builds oracle/_ref/libfcl_ref.so: the reference's own convex query engine
# (include/fcl/cvx_collide/*, compiled unmodified from where it lies) behind
# oracle/ref_driver.cpp, with oracle/eigen_shim standing in for Eigen.
# Needs the reference sources (REF_ROOT, default /root/reference); writes only
# into oracle/_ref/.  -ffp-contract=off keeps results identical to the
# restatement's on every host.
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
ref_root="${REF_ROOT:-/root/reference}"
if [ ! -d "$ref_root/include/fcl/cvx_collide" ]; then
  echo "reference sources not found at $ref_root; skipping oracle/_ref" >&2
  exit 0
fi
mkdir -p "$here/_ref"
g++ -O2 -std=c++17 -ffp-contract=off -DNDEBUG -fPIC -shared \
  -I "$here/eigen_shim" -I "$ref_root/include" \
  "$here/ref_driver.cpp" -o "$here/_ref/libfcl_ref.so" -lpthread
echo "built $here/_ref/libfcl_ref.so"
