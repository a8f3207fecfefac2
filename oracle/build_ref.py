"""Build recipe for the compiled reference oracle (test infrastructure only).

The reference's implicit-step sources compile with g++ after a handful of
mechanical portability fixes (the original project targets MSVC 2015).  This
script

1. copies the hot-path translation units and headers from the reference tree
   (the argument, else ``$OD_REFERENCE``, else ``reference/OpenDeformer`` in
   the directory that holds this repository) into
   ``oracle/_ref/src/`` -- a git-ignored build directory, never the product;
2. applies the portability fixes to that copy (never to the reference tree);
3. compiles it together with ``oracle/ref_harness.cpp`` (a C API written for
   this project) into ``oracle/_ref/libodref.so``.

When the reference tree is absent (a machine that only received this
repository) and ``oracle/_ref/src/`` already holds the patched copy, step 3 is
run on that copy, so the oracle can be rebuilt for another CPU architecture.

Fixes applied (each is a compile error under g++ 13 otherwise):

1. ``core/oder.h``: forward declarations of MemoryArena/MemoryPool use
   ``unsigned int Align``; the definitions use ``size_t``.
2. ``core/oder.h``: add standard headers MSVC pulled in implicitly.
3. ``core/memory.h``: move allocAligned/freeAligned/Initiation/Destory/
   Construct above MemoryArena (two-phase name lookup).
4. ``core/sparseMatrix.h``: rename friend-template parameters that shadow the
   enclosing class template's parameters.
5. ``core/sparseMatrix.h``: typo ``blockColumnEntries`` -> ``blockColumnOris``
   in the move constructor/assignment.
6. ``core/intergrator.h``: ``DampingForcer`` -> ``StaDampingForcer``;
   ``intergrator/nonlinearImplicitBackwardEuler.h``: add ``typename``.
7. compile with ``-DODER_CORE_DATASTRUCTURE_H`` so ``core/datastructure.h``
   (mesher-only templates that shadow ``T``) is skipped.
8. ``collision/intersection.cpp``: keep the plane-tetrahedron intersection and
   the barycentric coordinates; drop the tetrahedron-tetrahedron
   intersection after them and its mesher includes (the mesher's exact
   arithmetic uses MSVC-only in-class specialisations);
   ``collision/penaltyDampingForcer.cpp``: drop
   MeshMeshCollisionDampingForcer::addDampingMatrix, its only caller (it
   computes an intersection and adds nothing to the matrix).
9. ``core/allocator.h``: add ``template`` before the dependent member-template
   calls ``alloc->Alloc<value_type>`` / ``alloc->Dealloc<value_type>``.

No ``-ffast-math``: the oracle is defined as this IEEE-strict g++ build.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_OUT = os.path.join(HERE, "_ref")
SRC_OUT = os.path.join(REF_OUT, "src")
LIB_OUT = os.path.join(REF_OUT, "libodref.so")

FILES = {
    "core": ["oder.h", "memory.h", "memory.cpp", "latool.h", "latool.cpp",
             "sparseMatrix.h", "sparseMatrix.cpp", "numerMethod.h", "element.h",
             "mesh.h", "mesh.cpp", "nodeIndexer.h", "nodeIndexer.cpp",
             "constrainer.h", "constrainer.cpp", "forcer.h", "forcer.cpp",
             "mechMaterial.h", "mechMaterial.cpp", "intergrator.h",
             "linearSolver.h", "preconditioner.h", "simulator.h",
             "simulator.cpp", "stdafx.h", "datastructure.h", "allocator.h", "meshRelabeler.h",
             "meshRelabler.cpp"],
    "element": ["tetelement.h", "tetelement.cpp"],
    "mesh": ["tetmesh.h", "tetmesh.cpp"],
    "material": ["fullOrderNonlinear.h", "corotationalHyperelastic.h",
                 "corotationalHyperelastic.cpp", "invertibleHyperelastic.h",
                 "invertibleHyperelastic.cpp", "invertibleNeoHookean.h",
                 "invertibleNeoHookean.cpp", "invertibleStVK.h",
                 "invertibleStVK.cpp", "corotationalPlastic.h", "corotationalPlastic.cpp",
                 "hooke.h", "hooke.cpp"],
    "solver": ["cgSolver.h", "cgSolver.cpp", "jacobiPreconditioner.h",
               "jacobiPreconditioner.cpp", "inCholeskyPreconditioner.h",
               "inCholeskyPreconditioner.cpp", "inLDLTPreconditioner.h",
               "inLDLTPreconditioner.cpp"],
    "intergrator": ["nonlinearImplicitBackwardEuler.h"],
    "collision": ["collisionShapes.h", "intersection.h", "intersection.cpp", "penaltyDampingForcer.h",
                  "penaltyDampingForcer.cpp"],
}


def _replace(text: str, old: str, new: str, path: str, count: int = 1) -> str:
    n = text.count(old)
    if n != count:
        raise RuntimeError(f"patch anchor found {n}x (expected {count}) in {path}: {old[:60]!r}")
    return text.replace(old, new)


def _patch(root: str) -> None:
    def rw(rel, fn):
        p = os.path.join(root, rel)
        with open(p, "r", encoding="utf-8", errors="surrogateescape") as f:
            t = f.read()
        t = fn(t, p)
        with open(p, "w", encoding="utf-8", errors="surrogateescape") as f:
            f.write(t)

    def oder(t, p):
        t = _replace(t, "template<class T, unsigned int Align> class MemoryArena;",
                     "template<class T, size_t Align> class MemoryArena;", p)
        t = _replace(t, "template<class T, unsigned int Align> class MemoryPool;",
                     "template<class T, size_t Align> class MemoryPool;", p)
        t = _replace(t, "#include <string.h>\n",
                     "#include <string.h>\n#include <stdio.h>\n#include <limits>\n"
                     "#include <climits>\n#include <utility>\n#include <type_traits>\n"
                     "#include <tuple>\n", p)
        return t

    def memory(t, p):
        start_tok = "\ttemplate<size_t Align = ODER_L1_CACHE_LINE_SIZE> void *allocAligned(size_t size){"
        end_tok = "\t\tnew (p) T(std::forward<Args>(inits)...);\n\t}\n"
        s = t.index(start_tok)
        e = t.index(end_tok, s) + len(end_tok)
        block = t[s:e]
        t = t[:s] + t[e:]
        anchor = "\ttemplate<class T, size_t Align = std::alignment_of<T>::value> class MemoryArena{"
        t = _replace(t, anchor, block + "\n" + anchor, p)
        return t

    def sparse(t, p):
        t = _replace(t, "\t\ttemplate<int blockLength, int blockWidth>\n\t\tfriend void SpMDV(const BlockedSymSparseMatrix<blockLength, blockWidth>& mat,",
                     "\t\ttemplate<int bL, int bW>\n\t\tfriend void SpMDV(const BlockedSymSparseMatrix<bL, bW>& mat,", p)
        t = _replace(t, "\t\ttemplate<int blockLength, int blockWidth>\n\t\tfriend void SpMSV(const BlockedSymSparseMatrix<blockLength, blockWidth>& mat,",
                     "\t\ttemplate<int bL, int bW>\n\t\tfriend void SpMSV(const BlockedSymSparseMatrix<bL, bW>& mat,", p, count=2)
        t = _replace(t, "\t\ttemplate<class SpMatrix, int blockLength, int blockWidth>\n\t\tfriend void SpMDV(const AggregatedSparseMatrix<SpMatrix, blockLength, blockWidth>& mat,",
                     "\t\ttemplate<class SpM, int bL, int bW>\n\t\tfriend void SpMDV(const AggregatedSparseMatrix<SpM, bL, bW>& mat,", p)
        t = _replace(t, "blockColumnEntries = mat.blockColumnOris;", "blockColumnOris = mat.blockColumnOris;", p)
        t = _replace(t, "std::swap(blockColumnEntries, mat.blockColumnOris);", "std::swap(blockColumnOris, mat.blockColumnOris);", p)
        return t

    def integ(t, p):
        return _replace(t, "const DampingForcer& forcer", "const StaDampingForcer& forcer", p)

    def be(t, p):
        return _replace(t, "using AssemblerType = SpMatrix::Assembler;",
                        "using AssemblerType = typename SpMatrix::Assembler;", p)

    def intersection(t, p):
        # keep the plane-tetrahedron part; the tetrahedron-tetrahedron
        # intersection below it needs the mesher's exact arithmetic, which
        # does not compile under g++
        t = _replace(t, '#include "delPrimitive.h"\n#include "predicate.h"\n#include "geometer.h"\n', "", p)
        cut = t.index("\t\tvoid digCavity(")
        return t[:cut] + "\t}\n}\n"

    def damping(t, p):
        # MeshMeshCollisionDampingForcer::addDampingMatrix calls that
        # tetrahedron-tetrahedron intersection (and adds nothing)
        cut = t.index("\t\tvoid MeshMeshCollisionDampingForcer::addDampingMatrix")
        return t[:cut] + "\t}\n}\n"

    def allocator(t, p):
        t = _replace(t, "alloc->Alloc<value_type>(n)", "alloc->template Alloc<value_type>(n)", p)
        return _replace(t, "alloc->Dealloc<value_type>(p, n)", "alloc->template Dealloc<value_type>(p, n)", p)

    rw("core/oder.h", oder)
    rw("core/allocator.h", allocator)
    rw("collision/intersection.cpp", intersection)
    rw("collision/penaltyDampingForcer.cpp", damping)
    rw("core/memory.h", memory)
    rw("core/sparseMatrix.h", sparse)
    rw("core/intergrator.h", integ)
    rw("intergrator/nonlinearImplicitBackwardEuler.h", be)


def copy_and_patch(ref_root: str) -> None:
    if os.path.isdir(SRC_OUT):
        shutil.rmtree(SRC_OUT)
    for sub, names in FILES.items():
        os.makedirs(os.path.join(SRC_OUT, sub), exist_ok=True)
        for n in names:
            shutil.copyfile(os.path.join(ref_root, sub, n), os.path.join(SRC_OUT, sub, n))
    _patch(SRC_OUT)


def compile_lib(jobs: int = 8) -> str:
    inc = []
    for sub in FILES:
        inc += ["-I", os.path.join(SRC_OUT, sub)]
    flags = ["-std=c++17", "-O2", "-fPIC", "-DNDEBUG", "-DODER_CORE_DATASTRUCTURE_H",
             "-w", "-ffp-contract=off"]
    srcs = [os.path.join(SRC_OUT, sub, n) for sub, names in FILES.items() for n in names
            if n.endswith(".cpp")]
    srcs.append(os.path.join(HERE, "ref_harness.cpp"))
    objdir = os.path.join(REF_OUT, "obj")
    os.makedirs(objdir, exist_ok=True)
    procs, objs = [], []
    for s in srcs:
        o = os.path.join(objdir, os.path.basename(s) + ".o")
        objs.append(o)
        procs.append(subprocess.Popen(["g++", *flags, *inc, "-c", s, "-o", o]))
        if len(procs) >= jobs:
            if procs.pop(0).wait() != 0:
                raise RuntimeError("reference oracle compile failed")
    for p in procs:
        if p.wait() != 0:
            raise RuntimeError("reference oracle compile failed")
    subprocess.check_call(["g++", "-shared", "-o", LIB_OUT, *objs])
    return LIB_OUT


def build(ref_root: str | None = None) -> str | None:
    """Build ``oracle/_ref/libodref.so``; returns its path or None if impossible."""
    ref_root = ref_root or os.environ.get("OD_REFERENCE") or os.path.join(
        os.path.dirname(os.path.dirname(HERE)), "reference", "OpenDeformer")
    if os.path.isdir(ref_root):
        copy_and_patch(ref_root)
    elif not os.path.isdir(SRC_OUT):
        return None
    return compile_lib()


if __name__ == "__main__":
    out = build(sys.argv[1] if len(sys.argv) > 1 else None)
    print(out or "reference sources unavailable")
