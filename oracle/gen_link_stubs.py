"""Link stubs for the reference pin library (TEST INFRASTRUCTURE ONLY).

The reference's translation units on the pinned path (compiled unmodified
against oracle/shim/) also reference functions of the samplers, of waveform
models off the path and of GSL routines that no pinned call reaches.  This
script links the objects once with --no-undefined, reads the symbols the
linker reports as undefined, and writes a C file that defines each of them:
functions as stubs that print their name and abort, data symbols as zeroed
storage.  A pinned call that reached a stub would therefore stop loudly
instead of computing something else.

  python gen_link_stubs.py OUT.c -- <link command ...>
"""
import re
import subprocess
import sys

# C data symbols the shim headers declare extern (all other C names are functions)
C_DATA = {"gsl_rng_default", "gsl_min_fminimizer_brent"}


def main():
    out = sys.argv[1]
    cmd = sys.argv[sys.argv.index("--") + 1:]
    r = subprocess.run(cmd + ["-Wl,--no-undefined", "-Wl,--no-demangle"], capture_output=True, text=True)
    names = sorted(set(re.findall(r"undefined reference to `([^']+)'", r.stdout + r.stderr)))
    if r.returncode != 0 and not names:
        sys.stderr.write(r.stdout + r.stderr)
        sys.exit(1)
    dem = subprocess.run(["c++filt"], input="\n".join(names), capture_output=True, text=True).stdout.split("\n")
    lines = ["/* generated by oracle/gen_link_stubs.py: link stubs, never called on the pinned path */",
             "#include <stdio.h>", "#include <stdlib.h>",
             "static void gwo_stub_abort(const char *name) {",
             '  fprintf(stderr, "reference pin library: unpinned symbol %s was called\\n", name);',
             "  abort();", "}"]
    for i, (n, d) in enumerate(zip(names, dem)):
        if n in C_DATA:
            lines.append("const void *gwo_stub_data_%d __asm__(\"%s\");" % (i, n))
            lines.append("const void *gwo_stub_data_%d = 0;" % i)
        elif d.startswith(("vtable for", "typeinfo", "VTT for", "guard variable")):
            lines.append("char gwo_stub_data_%d[256] __asm__(\"%s\");" % (i, n))
            lines.append("char gwo_stub_data_%d[256];" % i)
        else:
            lines.append("void gwo_stub_%d(void) __asm__(\"%s\");" % (i, n))
            lines.append("void gwo_stub_%d(void) { gwo_stub_abort(\"%s\"); }" % (i, d.replace("\"", "'")))
    open(out, "w").write("\n".join(lines) + "\n")


if __name__ == "__main__":
    main()
