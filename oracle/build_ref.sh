#!/usr/bin/env bash
# Recipe that compiles the reference (mind-fcl) from its own sources, where
# they lie, into oracle/_ref/ — test infrastructure only:
#   libfcl_ref.so       the convex query engine (include/fcl/cvx_collide/*)
#                       behind oracle/ref_driver.cpp, with oracle/eigen_shim;
#   libfcl_ref_mesh.so  BVHModel<OBBRSS>, MeshIntersect and the closed-form
#                       shape solvers behind oracle/ref_mesh_driver.cpp, with
#                       the general oracle/eigen_shim_full.
# The reference headers are compiled unmodified; the shims are this project's
# own stand-ins for Eigen, which the reference needs and which is absent here.
# REF_ROOT selects the reference checkout (this recipe's default is the
# container's read-only copy); where it holds no sources the recipe does
# nothing.  Writes only into oracle/_ref/.  -ffp-contract=off keeps results
# identical to the restatements' on every host.
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
ref_root="${REF_ROOT:-/root/reference}"
if [ ! -d "$ref_root/include/fcl/cvx_collide" ]; then
  echo "reference sources not found; skipping oracle/_ref" >&2
  exit 0
fi
mkdir -p "$here/_ref"
build() {  # out driver shim
  local out="$here/_ref/$1" src="$here/$2" shim="$here/$3"
  if [ -f "$out" ] && [ -z "$(find "$src" "$shim" -newer "$out" -type f)" ]; then
    return 0
  fi
  g++ -O2 -std=c++17 -ffp-contract=off -DNDEBUG -fPIC -shared \
    -I "$shim" -I "$ref_root/include" "$src" -o "$out" -lpthread
  echo "built $out"
}
build libfcl_ref.so ref_driver.cpp eigen_shim &
build libfcl_ref_mesh.so ref_mesh_driver.cpp eigen_shim_full &
wait %1
wait %2
