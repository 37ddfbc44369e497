#define GITVERSION "oracle-build"
