// Times the reference's sequential Dijkstra (seqSSSPwithDist_undir.cpp, djk, SEQ:66-180) on
// one graph file, for comparing the oracle restatement that the benchmark's CPU baseline
// runs against the reference's own compiled code.  Test infrastructure; built by
// `make -C oracle ref` from the reference's sources where they lie (nothing is copied).
//
//   ref_time <graph file> <nodes> <source>
// prints "<seconds of djk> <checksum of the printed distances>" on stdout.  The read
// (readin_graphU2) is not timed; djk's own print loop is (the reference times it that way
// too when run as a program), with cout sent to a buffer that discards and sums what it gets.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <streambuf>

#define main reference_seq_main
#include "seqSSSPwithDist_undir.cpp"
#undef main

namespace {

// Discards what is written and keeps a checksum of the characters.
class SumBuf : public std::streambuf {
  public:
    unsigned long long sum = 0;

  protected:
    int overflow(int c) override {
        if (c != EOF) sum = sum * 131 + (unsigned char)c;
        return c;
    }
};

}  // namespace

int main(int argc, char* argv[]) {
    if (argc < 4) {
        fprintf(stderr, "usage: ref_time <graph file> <nodes> <source>\n");
        return 2;
    }
    const int nodes = atoi(argv[2]), src = atoi(argv[3]);
    A_Network X, Y;
    ADJ_Bundle adjobj;
    X.resize(nodes, adjobj);
    Y.resize(nodes, adjobj);
    readin_graphU2(&X, nodes, argv[1]);
    SumBuf sink;
    std::streambuf* old = cout.rdbuf(&sink);
    const auto t0 = std::chrono::steady_clock::now();
    djk(src, &X, &Y, nodes);
    const auto t1 = std::chrono::steady_clock::now();
    cout.rdbuf(old);
    printf("%.6f %llu\n", std::chrono::duration<double>(t1 - t0).count(), sink.sum);
    return 0;
}
