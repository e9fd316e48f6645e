/*
 * ref_shim.cpp — driver for the UNMODIFIED reference C model
 * (Range_Limited_demo/SourceCode/C_Model_ForceEval/MD_Evaluation_Model.cpp), built by
 * oracle/build_ref.sh into oracle/_ref/.  Test infrastructure only.
 *
 * The reference opens a hard-coded absolute path ending in "ar_gas.pdb" (.cpp:30-39).  This
 * shim supplies main() and interposes fopen/fopen64 (which std::ifstream calls inside libstdc++)
 * so that the path is redirected to the file named by MDRL_REF_PDB; every other open passes
 * through unchanged.  The reference's source is compiled as it lies.
 */
#include <dlfcn.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

int MD_Evaluation_Model();

static const char *redirect(const char *path) {
    const char *want = "ar_gas.pdb";
    const size_t n = strlen(path), m = strlen(want);
    const char *to = getenv("MDRL_REF_PDB");
    if (to && n >= m && strcmp(path + n - m, want) == 0) return to;
    return path;
}

extern "C" FILE *fopen(const char *path, const char *mode) {
    typedef FILE *(*fn_t)(const char *, const char *);
    static fn_t real = (fn_t)dlsym(RTLD_NEXT, "fopen");
    return real(redirect(path), mode);
}

extern "C" FILE *fopen64(const char *path, const char *mode) {
    typedef FILE *(*fn_t)(const char *, const char *);
    static fn_t real = (fn_t)dlsym(RTLD_NEXT, "fopen64");
    return real(redirect(path), mode);
}

int main() { return MD_Evaluation_Model() == 1 ? 0 : 1; }
