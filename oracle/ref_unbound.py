"""Writes _ref/unbound.cpp for oracle/ref.mk: one definition for each symbol
that the compiled reference objects use but none of them defines and the C,
C++ and math runtimes do not provide (the parts of the reference solver
outside the checked path).  Functions abort with their name when called;
variables get zeroed storage.  Test infrastructure only.

usage: python3 ref_unbound.py OUT.cpp OBJ...
"""
import subprocess
import sys


def symbols(args):
    out = subprocess.run(["nm"] + args, capture_output=True, text=True, check=True).stdout
    return out.split("\n")


def runtime_symbols():
    """Symbols a plain g++ link against libstdc++, libm and libc resolves."""
    probe = subprocess.run(["g++", "-print-file-name=libstdc++.so"], capture_output=True, text=True).stdout.strip()
    libs = [probe]
    for name in ("libc.so.6", "libm.so.6", "libgcc_s.so.1"):
        p = subprocess.run(["g++", "-print-file-name=" + name], capture_output=True, text=True).stdout.strip()
        libs.append(p)
    have = set()
    for lib in libs:
        r = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True, text=True)
        for line in r.stdout.split("\n"):
            parts = line.split()
            if len(parts) >= 3:
                have.add(parts[2].split("@")[0])
    return have


def demangle(names):
    if not names:
        return []
    out = subprocess.run(["c++filt"], input="\n".join(names), capture_output=True, text=True, check=True).stdout
    return out.split("\n")[: len(names)]


def main():
    dst, objs = sys.argv[1], sys.argv[2:]
    undefined, defined = set(), set()
    for line in symbols(objs):
        parts = line.split()
        if len(parts) == 2 and parts[0] == "U":
            undefined.add(parts[1])
        elif len(parts) == 3 and parts[1] not in ("U", "w", "v"):
            defined.add(parts[2])
    runtime = runtime_symbols()
    missing = sorted(s for s in undefined - defined if s not in runtime and not s.startswith("__")
                     and not s.startswith("_GLOBAL_OFFSET"))
    pretty = demangle(missing)
    lines = ["// Generated by ref_unbound.py: symbols outside the checked path.",
             "int vfs_ref_unimpl(const char*);", "extern \"C\" {"]
    for sym, dm in zip(missing, pretty):
        if "(" in dm:  # a function
            text = dm.replace("\\", "\\\\").replace('"', '\\"')
            lines.append(f'void {sym}() {{ vfs_ref_unimpl("{text}"); }}')
        else:  # a variable declared by the reference's headers, defined elsewhere
            lines.append(f"__attribute__((aligned(64))) char {sym}[4096];")
    lines.append("}")
    with open(dst, "w") as f:
        f.write("\n".join(lines) + "\n")
    print(f"ref_unbound: {len(missing)} symbols bound to stubs", file=sys.stderr)


if __name__ == "__main__":
    main()
