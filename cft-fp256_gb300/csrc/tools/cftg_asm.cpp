// cftg-asm - the `.cfta` assembler as a command, over libcft_gb300's
// cftg_asm_* calls. The command lines of the reference's host/tools/cft-asm
// (assemble, -d disassemble, -i header report), plus --bank for the ODE
// programs' default banks (programs/gen_odes.py:bank_values):
//
//   cftg-asm kernel.cfta -o kernel.cftp         assemble (no -o: check only)
//   cftg-asm -d kernel.cftp                     disassemble to stdout
//   cftg-asm -i kernel.cftp                     the header and the SHA-256
//   cftg-asm --bank SYSTEM FORMAT H -o x.bank   an ODE bank for step H
//
// Exit status 0 on success, 1 on a refusal (the reason on stderr).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../../include/cft_gb300.h"

static int usage(FILE *f)
{
    fprintf(f,
            "usage: cftg-asm SOURCE.cfta [-o IMAGE.cftp]\n"
            "       cftg-asm -d IMAGE.cftp\n"
            "       cftg-asm -i IMAGE.cftp\n"
            "       cftg-asm --bank lorenz63-rk4|lorenz96-rk4|henonheiles-lf fp32|fp64|fp128|fp256 H -o OUT.bank\n");
    return f == stdout ? 0 : 1;
}

static bool read_file(const char *path, std::string *out)
{
    FILE *f = fopen(path, "rb");
    if (!f) return false;
    char buf[65536];
    size_t n;
    while ((n = fread(buf, 1, sizeof buf, f)) > 0) out->append(buf, n);
    const bool ok = !ferror(f);
    fclose(f);
    return ok;
}

static bool write_file(const char *path, const void *p, size_t n)
{
    FILE *f = fopen(path, "wb");
    if (!f) return false;
    const bool ok = fwrite(p, 1, n, f) == n;
    return (fclose(f) == 0) && ok;
}

static int refuse(const char *what)
{
    fprintf(stderr, "cftg-asm: %s\n", what);
    return 1;
}

int main(int argc, char **argv)
{
    const char *in = nullptr, *out = nullptr;
    char mode = 'a';
    std::vector<const char *> bank;
    for (int i = 1; i < argc; i++) {
        const char *a = argv[i];
        if (!strcmp(a, "-h") || !strcmp(a, "--help")) return usage(stdout);
        if (!strcmp(a, "-d")) mode = 'd';
        else if (!strcmp(a, "-i")) mode = 'i';
        else if (!strcmp(a, "-o")) {
            if (i + 1 >= argc) return refuse("-o needs a path");
            out = argv[++i];
        } else if (!strcmp(a, "--bank")) {
            if (i + 3 >= argc) return refuse("--bank needs SYSTEM FORMAT H");
            mode = 'b';
            bank = {argv[i + 1], argv[i + 2], argv[i + 3]};
            i += 3;
        } else if (a[0] == '-' && a[1]) {
            fprintf(stderr, "cftg-asm: unknown option %s\n", a);
            return 1;
        } else {
            if (in) return refuse("one input file at a time");
            in = a;
        }
    }
    if (mode == 'b') {
        int fmt = -1;
        static const char *const names[4] = {"fp32", "fp64", "fp128", "fp256"};
        for (int f = 0; f < 4; f++)
            if (!strcmp(bank[1], names[f])) fmt = f;
        if (fmt < 0) return refuse("FORMAT is fp32, fp64, fp128 or fp256");
        if (!out) return refuse("--bank needs -o OUT.bank");
        size_t need = 0;
        if (cftg_ode_bank(bank[0], (cft_format)fmt, bank[2], nullptr, 0, &need) != CFT_OK)
            return refuse(cft_last_error());
        std::vector<unsigned char> b(need);
        if (cftg_ode_bank(bank[0], (cft_format)fmt, bank[2], b.data(), b.size(), &need) != CFT_OK)
            return refuse(cft_last_error());
        if (!write_file(out, b.data(), b.size())) return refuse("cannot write the bank");
        return 0;
    }
    if (!in) return usage(stderr);
    std::string data;
    if (!read_file(in, &data)) {
        fprintf(stderr, "cftg-asm: cannot read %s\n", in);
        return 1;
    }
    if (mode == 'a') {
        void *img = nullptr;
        size_t n = 0;
        if (cftg_asm_assemble(data.data(), data.size(), in, &img, &n) != CFT_OK)
            return refuse(cft_last_error());
        const bool ok = !out || write_file(out, img, n);
        cftg_asm_free(img);
        if (!ok) {
            fprintf(stderr, "cftg-asm: cannot write %s\n", out);
            return 1;
        }
        return 0;
    }
    char *text = nullptr;
    const cft_status st = mode == 'd' ? cftg_asm_disassemble(data.data(), data.size(), &text)
                                      : cftg_asm_info(data.data(), data.size(), &text);
    if (st != CFT_OK) return refuse(cft_last_error());
    fputs(text, stdout);
    cftg_asm_free(text);
    return 0;
}
