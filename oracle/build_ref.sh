#!/bin/sh
# Recipe: builds oracle/_ref/libvor3d_ref.so (the reference's own vor3d core,
# compiled unmodified, used only to pin the oracle) from the reference source
# tree where it exists. VO_REF_ROOT overrides the location; without the
# sources (e.g. on a machine that only runs the GPU tests) it does nothing.
REF_ROOT="${VO_REF_ROOT:-/root/reference}"
[ -d "$REF_ROOT/src/vor3d" ] || exit 0
exec make -s -C "$(dirname "$0")" ref REF_ROOT="$REF_ROOT"
