// Thread-MPI shim -- TEST INFRASTRUCTURE ONLY (part of the oracle).
// Implements the declarations of mpi.h in this folder: P thread-ranks sharing
// one process, eager sends into per-rank mailboxes, receives matched on
// (source, tag) in arrival order.
#include "mpi.h"

#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <vector>

struct tmpi_comm_s {
    tmpi_world *world;
    int rank;
};

struct tmpi_message {
    int source;
    int tag;
    std::vector<unsigned char> payload;
};

struct tmpi_request_s {
    bool is_recv;
    void *buf;
    size_t bytes;
    int peer;
    int tag;
    tmpi_comm_s *comm;
};

struct tmpi_world_s {
    int n_ranks;
    std::vector<tmpi_comm_s> comms;
    std::mutex mu;
    std::condition_variable cv;
    std::vector<std::deque<tmpi_message>> mailbox; // indexed by receiver
    // barrier state
    int barrier_count = 0;
    unsigned long barrier_generation = 0;
};

extern "C" {

size_t tmpi_type_size(MPI_Datatype type) {
    switch (type) {
    case MPI_CHAR:
    case MPI_UNSIGNED_CHAR:
    case MPI_CXX_BOOL:
        return 1;
    case MPI_SHORT:
        return 2;
    case MPI_INT:
    case MPI_UINT32_T:
    case MPI_FLOAT:
        return 4;
    case MPI_UNSIGNED_LONG:
    case MPI_UNSIGNED_LONG_LONG:
    case MPI_DOUBLE:
    case MPI_CXX_FLOAT_COMPLEX:
        return 8;
    case MPI_CXX_DOUBLE_COMPLEX:
        return 16;
    default:
        return 0;
    }
}

tmpi_world *tmpi_world_create(int n_ranks) {
    if (n_ranks <= 0)
        return nullptr;
    tmpi_world *w = new tmpi_world();
    w->n_ranks = n_ranks;
    w->comms.resize(n_ranks);
    for (int r = 0; r < n_ranks; ++r)
        w->comms[r] = tmpi_comm_s{w, r};
    w->mailbox.resize(n_ranks);
    return w;
}

void tmpi_world_destroy(tmpi_world *w) { delete w; }

MPI_Comm tmpi_comm(tmpi_world *w, int rank) {
    if (!w || rank < 0 || rank >= w->n_ranks)
        return nullptr;
    return &w->comms[rank];
}

size_t tmpi_world_pending_bytes(tmpi_world *w) {
    std::lock_guard<std::mutex> lk(w->mu);
    size_t total = 0;
    for (auto &box : w->mailbox)
        for (auto &m : box)
            total += m.payload.size();
    return total;
}

int MPI_Comm_rank(MPI_Comm comm, int *rank) {
    *rank = comm->rank;
    return MPI_SUCCESS;
}

int MPI_Comm_size(MPI_Comm comm, int *size) {
    *size = comm->world->n_ranks;
    return MPI_SUCCESS;
}

int MPI_Isend(const void *buf, int count, MPI_Datatype type, int dest, int tag,
              MPI_Comm comm, MPI_Request *req) {
    tmpi_world *w = comm->world;
    if (dest < 0 || dest >= w->n_ranks || count < 0)
        return MPI_ERR_OTHER;
    size_t bytes = (size_t)count * tmpi_type_size(type);
    tmpi_message m;
    m.source = comm->rank;
    m.tag = tag;
    m.payload.resize(bytes);
    if (bytes)
        std::memcpy(m.payload.data(), buf, bytes);
    {
        std::lock_guard<std::mutex> lk(w->mu);
        w->mailbox[dest].push_back(std::move(m));
    }
    w->cv.notify_all();
    // eager: the send is complete once the payload sits in the mailbox
    *req = new tmpi_request_s{false, nullptr, bytes, dest, tag, comm};
    return MPI_SUCCESS;
}

int MPI_Irecv(void *buf, int count, MPI_Datatype type, int source, int tag,
              MPI_Comm comm, MPI_Request *req) {
    if (source < 0 || source >= comm->world->n_ranks || count < 0)
        return MPI_ERR_OTHER;
    size_t bytes = (size_t)count * tmpi_type_size(type);
    *req = new tmpi_request_s{true, buf, bytes, source, tag, comm};
    return MPI_SUCCESS;
}

// Tries to complete `r` with the mailbox lock held; true when done.
static bool try_complete_locked(tmpi_request_s *r, MPI_Status *status) {
    if (!r->is_recv)
        return true;
    tmpi_world *w = r->comm->world;
    auto &box = w->mailbox[r->comm->rank];
    for (auto it = box.begin(); it != box.end(); ++it) {
        if (it->source == r->peer && it->tag == r->tag) {
            size_t n = it->payload.size() < r->bytes ? it->payload.size() : r->bytes;
            if (n)
                std::memcpy(r->buf, it->payload.data(), n);
            if (status) {
                status->MPI_SOURCE = it->source;
                status->MPI_TAG = it->tag;
                status->MPI_ERROR = MPI_SUCCESS;
            }
            box.erase(it);
            return true;
        }
    }
    return false;
}

int MPI_Wait(MPI_Request *req, MPI_Status *status) {
    if (!*req)
        return MPI_SUCCESS;
    tmpi_world *w = (*req)->comm->world;
    std::unique_lock<std::mutex> lk(w->mu);
    while (!try_complete_locked(*req, status))
        w->cv.wait(lk);
    delete *req;
    *req = MPI_REQUEST_NULL;
    return MPI_SUCCESS;
}

int MPI_Waitany(int count, MPI_Request reqs[], int *index, MPI_Status *status) {
    tmpi_world *w = nullptr;
    for (int i = 0; i < count; ++i)
        if (reqs[i]) {
            w = reqs[i]->comm->world;
            break;
        }
    if (!w) {
        *index = MPI_UNDEFINED;
        return MPI_SUCCESS;
    }
    std::unique_lock<std::mutex> lk(w->mu);
    for (;;) {
        for (int i = 0; i < count; ++i) {
            if (reqs[i] && try_complete_locked(reqs[i], status)) {
                delete reqs[i];
                reqs[i] = MPI_REQUEST_NULL;
                *index = i;
                return MPI_SUCCESS;
            }
        }
        w->cv.wait(lk);
    }
}

int MPI_Waitall(int count, MPI_Request reqs[], MPI_Status statuses[]) {
    for (int i = 0; i < count; ++i) {
        int rc = MPI_Wait(&reqs[i], statuses ? &statuses[i] : MPI_STATUS_IGNORE);
        if (rc != MPI_SUCCESS)
            return rc;
    }
    return MPI_SUCCESS;
}

int MPI_Barrier(MPI_Comm comm) {
    tmpi_world *w = comm->world;
    std::unique_lock<std::mutex> lk(w->mu);
    unsigned long gen = w->barrier_generation;
    if (++w->barrier_count == w->n_ranks) {
        w->barrier_count = 0;
        ++w->barrier_generation;
        w->cv.notify_all();
        return MPI_SUCCESS;
    }
    while (gen == w->barrier_generation)
        w->cv.wait(lk);
    return MPI_SUCCESS;
}

double MPI_Wtime(void) {
    using clk = std::chrono::steady_clock;
    return std::chrono::duration<double>(clk::now().time_since_epoch()).count();
}

} // extern "C"
