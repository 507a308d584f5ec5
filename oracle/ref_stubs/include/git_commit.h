// Stand-in for the CMake-generated commit header of the reference build.
#ifndef WF_ORACLE_GIT_COMMIT_STUB_H
#define WF_ORACLE_GIT_COMMIT_STUB_H
#define GIT_COMMIT_HASH "oracle-build"
#endif
