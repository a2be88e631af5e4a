/*
 * modules.c -- the reference's module loader (src/voxrnd/modules.c:1-69) and
 * data-file search (src/voxtrees/datareader.c:88-125).
 *
 * A module is a shared object `<name>.so` whose `module_init()` returns a
 * struct vox_module {type, methods}; camera classes other than the two
 * built-in ones come this way (camera.c:43-48).  It is looked for in the
 * module directory this library was built with (VOX_MODULE_PATH, none by
 * default) and then in $VOXVISION_MODULES, and opened with RTLD_NODELETE so
 * that its methods stay valid after the handle is closed, as the reference
 * does.  Data files are looked for as given, in VOX_DATA_PATH (none by
 * default) and in $VOXVISION_DATA, which the reference sets to
 * $HOME/.voxvision when unset (datareader.c:95-103); here that default is
 * applied by the lookup instead of by changing the environment at load.
 */
#include <dlfcn.h>
#include <limits.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>

#include "../../include/voxrnd.h"

#define EXPORT __attribute__((visibility("default")))

#ifndef VOX_MODULE_PATH
#define VOX_MODULE_PATH ""
#endif
#ifndef VOX_DATA_PATH
#define VOX_DATA_PATH ""
#endif

static int regular_file(const char *path)
{
    struct stat sb;
    return stat(path, &sb) == 0 && S_ISREG(sb.st_mode);
}

/* `dir` + `sep` + `name` + `ext` into out (PATH_MAX bytes); 0 if it does not fit. */
static int join(char *out, const char *dir, const char *sep, const char *name, const char *ext)
{
    int n = snprintf(out, PATH_MAX, "%s%s%s%s", dir, sep, name, ext);
    return n >= 0 && n < PATH_MAX;
}

/* modules.c:23-41 */
static int find_module(const char *name, char *path)
{
    if (VOX_MODULE_PATH[0] && join(path, VOX_MODULE_PATH, "", name, ".so") && regular_file(path)) return 1;
    const char *env = getenv("VOXVISION_MODULES");
    if (env && join(path, env, "/", name, ".so") && regular_file(path)) return 1;
    return 0;
}

/* modules.c:43-69 */
EXPORT struct vox_module_methods *vox_load_module(const char *name, int type)
{
    char path[PATH_MAX];
    if (!name || !find_module(name, path)) return NULL;
    void *handle = dlopen(path, RTLD_LAZY | RTLD_NODELETE);
    if (!handle) return NULL;
    struct vox_module *(*module_init)(void);
    *(void **)&module_init = dlsym(handle, "module_init");
    dlclose(handle);   /* RTLD_NODELETE: the code stays mapped */
    if (!module_init) return NULL;
    struct vox_module *module = module_init();
    if (!module || module->type != type) return NULL;
    return module->methods;
}

/* datareader.c:105-125 */
EXPORT int vox_find_data_file(const char *filename, char *fullpath)
{
    if (!filename || !fullpath) return 0;
    if (join(fullpath, filename, "", "", "") && regular_file(fullpath)) return 1;
    if (VOX_DATA_PATH[0] && join(fullpath, VOX_DATA_PATH, "", filename, "") && regular_file(fullpath)) return 1;
    const char *env = getenv("VOXVISION_DATA");
    char home[PATH_MAX];
    if (!env) {
        const char *h = getenv("HOME");
        if (h && join(home, h, "/", ".voxvision", "")) env = home;
    }
    if (env && join(fullpath, env, "/", filename, "") && regular_file(fullpath)) return 1;
    return 0;
}
