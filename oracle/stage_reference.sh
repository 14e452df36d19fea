#!/bin/sh
# Stages the reference BWA fork's sources for builds on machines that have no
# BSBolt checkout (the GPU host): copies bsbolt/External/BWA of the checkout at
# $BSB_REFERENCE (default /root/reference) into baseline/_ref/bwa, which is
# git-ignored and travels with the working tree.  The copy is only read by
# oracle/Makefile.ref (the stock `bwa`, the reference's CPU baseline and test
# oracle) and bsbolt_gb300/integration/Makefile (`bwa_gpu`); it is never
# committed.  Without a checkout, an existing copy is left as it is.
# Run from the repository root.
set -e
SRC="${BSB_REFERENCE:-/root/reference}/bsbolt/External/BWA"
DST=baseline/_ref/bwa
if [ -d "$SRC" ]; then
    mkdir -p "$DST"
    cp -p -u "$SRC"/*.c "$SRC"/*.h "$SRC"/*.cpp "$SRC"/COPYING "$DST"/
fi
[ -f "$DST/bwamem.c" ] || { echo "stage_reference: no BWA sources at $SRC or $DST" >&2; exit 1; }
